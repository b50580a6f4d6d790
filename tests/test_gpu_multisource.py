"""Multi-source dropout concealment through the chd_* ABI on the GPU.

A primary capture and extra captures of the same pictures -- their own noise
and dropouts, CAV picture numbers in the VBI (one extra starting a frame
later, one without VBI and aligned positionally, one ending early), VITS
bPSNR qualities -- are written as .tbc + JSON sidecars, attached with
chd_video_add_extra_source_composite and decoded with concealment on. Every
frame must match the oracle's multi-source decode (its extras aligned by the
oracle's own restatement of MultiSourceAlignment) within +-1 LSB, and the
dropout statistics exactly; the extras freeze on the first correcting decode
(src/abi/c_api_video.cpp:859-869)."""
import ctypes as C
import json

import numpy as np
import pytest

from libchromadec_gb300 import abi, synth
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NF = 16
SEED = 41


def _cav(pic):
    return [0, 0xF00000 | int(str(pic), 16), 0]


def _recapture(noise_seed, dropout_seed, dropouts, nfields=NF):
    cfg = synth.SynthConfig(seed=SEED, pan_x=1.5, pan_y=0.5, dropout_line_fraction=dropouts, noise_seed=noise_seed,
                            dropout_seed=dropout_seed)
    return synth.make_capture(nfields, cfg)


@pytest.fixture(scope="module")
def sources(tmp_path_factory):
    d = tmp_path_factory.mktemp("ms")
    rng = np.random.default_rng(5)
    prim = _recapture(None, None, 0.03)
    # extra A: the same disc from picture 301 on (the primary's frame 1 onwards)
    a_full = _recapture(91, 92, 0.04)
    a = synth.SynthCapture(fields=np.ascontiguousarray(a_full.fields[2:]), dropouts=a_full.dropouts[2:])
    # extra B: no VBI codes, positional, better quality
    b = _recapture(93, 94, 0.03)
    # extra C: VBI, ends two frames early
    c_full = _recapture(95, 96, 0.05)
    c = synth.SynthCapture(fields=np.ascontiguousarray(c_full.fields[:NF - 4]), dropouts=c_full.dropouts[:NF - 4])
    out = {}
    specs = {
        "prim": (prim, [_cav(300 + i // 2) for i in range(NF)], rng.uniform(30, 40, NF)),
        "a": (a, [_cav(301 + i // 2) for i in range(NF - 2)], np.full(NF - 2, 41.0)),
        "b": (b, None, np.full(NF, 44.0)),
        "c": (c, [_cav(300 + i // 2) for i in range(NF - 4)], np.full(NF - 4, 41.0)),
    }
    for name, (cap, vbi, bp) in specs.items():
        path = str(d / f"{name}.tbc")
        synth.write_tbc(path, cap, vbi=vbi, bpsnr=bp)
        out[name] = (path, cap, vbi, bp)
    return out


def _oracle_extras(sources, names):
    def meta(name):
        path, cap, vbi, bp = sources[name]
        m = json.load(open(path + ".json"))
        return ([f["isFirstField"] for f in m["fields"]],
                [tuple(f.get("vbi", {}).get("vbiData", [0, 0, 0])) for f in m["fields"]], True, True)

    frame_for = O.align_sources([meta("prim")] + [meta(n) for n in names])
    extras = []
    for s, name in enumerate(names, start=1):
        path, cap, vbi, bp = sources[name]
        nfr = cap.fields.shape[0] // 2
        fmap = []
        for f in range(NF // 2):
            k = frame_for(f + 1, s)
            fmap.append(k - 1 if 1 <= k <= nfr else -1)
        extras.append(dict(fields=cap.fields, dropouts=O.flatten_dropouts(cap.dropouts), bpsnr=bp, frame_map=fmap))
    return extras


def _compare(got, ref):
    d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
    assert d.max() <= 1, (d.max(), (d > 0).mean())


@pytest.mark.parametrize("kind,overcorrect,intra", [(3, False, False), (3, True, False), (2, False, True)])
def test_multi_source_concealment_matches_oracle(cuda, sources, kind, overcorrect, intra):
    names = ["a", "b", "c"]
    ppath, pcap, _, pbp = sources["prim"]
    v = abi.Video(ppath)
    L = abi.lib()
    for n in names:
        assert L.chd_video_add_extra_source_composite(v._h, sources[n][0].encode(), None) == 0
    # the library's alignment is the oracle's
    extras = _oracle_extras(sources, names)
    o = C.c_int32()
    for s, e in enumerate(extras, start=1):
        for f in range(NF // 2):
            assert L.chdg_video_source_frame(v._h, 0, s, f, C.byref(o)) == 0 and o.value == e["frame_map"][f]
    assert extras[0]["frame_map"][:3] == [-1, 0, 1] and extras[1]["frame_map"][:2] == [0, 1]
    assert extras[2]["frame_map"][-2:] == [-1, -1]
    d = abi.Decoder(v, abi.DEC_TRANSFORM_3D if kind == 3 else abi.DEC_TRANSFORM_2D)
    d.set("output_format", "yuv444p16")
    d.commit()
    d.set_dropout(True, overcorrect, intra)
    p = O.params(kind, O.FMT_P16)
    flat = O.flatten_dropouts(pcap.dropouts)
    ref, _ = O.decode_frames(p, pcap.fields, 0, NF // 2, dropouts=flat, overcorrect=overcorrect, intra=intra,
                             threads=8, bpsnr=pbp, extras=extras)
    single, _ = O.decode_frames(p, pcap.fields, 0, NF // 2, dropouts=flat, overcorrect=overcorrect, intra=intra,
                                threads=8)
    assert not np.array_equal(ref, single)   # the extras change the concealment
    for k in range(NF // 2):
        _, st = O.decode_frames(p, pcap.fields, k, 1, dropouts=flat, overcorrect=overcorrect, intra=intra,
                                threads=1, bpsnr=pbp, extras=extras)
        f = d.decode(k)
        _compare(f.planes(), ref[k])
        assert d.last_dropout_stats() == tuple(st), k
        f.close()
    # asynchronous path, same frames
    got = {i: pl for s, i, pl in d.decode_async(list(range(NF // 2)))}
    for k in range(NF // 2):
        _compare(got[k], ref[k])
    # the first correcting decode froze the extras
    assert L.chd_video_add_extra_source_composite(v._h, sources["b"][0].encode(), None) == abi.E_INVALID_ARG
    assert b"already run" in L.chd_last_error()


@pytest.mark.parametrize("overcorrect,intra", [(False, False), (True, False), (False, True)])
def test_multi_source_concealed_fields_byte_for_byte(cuda, sources, overcorrect, intra):
    """The concealed composite itself, replacement lines drawn from the extra
    captures, sample for sample against the oracle's multi-source corrector."""
    names = ["a", "b", "c"]
    ppath, pcap, _, pbp = sources["prim"]
    v = abi.Video(ppath)
    L = abi.lib()
    for n in names:
        assert L.chd_video_add_extra_source_composite(v._h, sources[n][0].encode(), None) == 0
    extras = _oracle_extras(sources, names)
    d = abi.Decoder(v, abi.DEC_TRANSFORM_3D)
    d.commit()
    d.set_dropout(True, overcorrect, intra)
    p = O.params(3, O.FMT_P16)
    flat = O.flatten_dropouts(pcap.dropouts)
    from_extras = 0
    for k in range(NF // 2):
        got = d.concealed_fields(k)
        ref, _ = O.dropout_correct_frame(p, pcap.fields, k, flat, overcorrect=overcorrect, intra=intra,
                                         bpsnr=pbp, extras=extras)
        single, _ = O.dropout_correct_frame(p, pcap.fields, k, flat, overcorrect=overcorrect, intra=intra)
        bad = np.argwhere(got != ref)
        assert bad.size == 0, (k, bad[:5])
        from_extras += int((ref != single).sum())
    assert from_extras > 0                                # some lines came from the extras
