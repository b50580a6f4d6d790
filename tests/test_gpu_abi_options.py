"""GPU parity of the widened decoder surface through the chd_* ABI:
CHD_DEC_PAL_2D (and AUTO, which resolves to it for PAL), luma noise coring,
the RGB and gray output formats with colour precisions, reverse_field_order
and subcarrier-locked captures; plus the device-level field-parity swap.
Each is compared with the CPU oracle, which reproduces the reference's own
code byte for byte on these options (tests/golden).

Tolerances: 16-bit formats within +-1 LSB (rgb48 truncates like the
reference, so a last-bit FP32 difference can move a sample by one code),
float formats within 1e-4; dropout statistics and spans bit-exact.
"""
import json

import numpy as np
import pytest

from libchromadec_gb300 import abi, synth
from oracle import oracle as O
from tests._capture import capture

pytestmark = pytest.mark.gpu

NF = 16
FMTS = {"yuv444p16": O.FMT_P16, "yuv444ps": O.FMT_PS, "rgb48": O.FMT_RGB48, "rgbs": O.FMT_RGBS,
        "gray16": O.FMT_GRAY16, "grays": O.FMT_GRAYS}


def _compare(got, ref, fmt):
    assert got.shape == ref.shape, (got.shape, ref.shape)
    if fmt in ("yuv444ps", "rgbs", "grays"):
        err = np.abs(got.astype(np.float64) - ref.astype(np.float64)).max()
        assert err < 1e-4, err
    else:
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 1, (d.max(), (d > 0).mean())


def _write(tmp_path, cap, name="cap.tbc", sc_locked=False):
    path = str(tmp_path / name)
    jpath = synth.write_tbc(path, cap)
    if sc_locked:
        meta = json.load(open(jpath))
        meta["videoParameters"]["isSubcarrierLocked"] = True
        json.dump(meta, open(jpath, "w"))
    return path


def _decode_all(path, kind, fmt="yuv444p16", dropout=None, **opts):
    v = abi.Video(path)
    d = abi.Decoder(v, kind)
    d.set("output_format", fmt)
    for k, val in opts.items():
        d.set(k, val)
    d.commit()
    if dropout is not None:
        d.set_dropout(True, *dropout)
    n = d.output_info().num_frames
    out, stats = [], []
    for k in range(n):
        f = d.decode(k)
        out.append(f.planes())
        stats.append(d.last_dropout_stats())
        f.close()
    return np.stack(out), stats, d, v


def _oracle_frames(p, fields, n, drops=None, oc=False, intra=False):
    frames, stats = [], []
    for k in range(n):
        out, st = O.decode_frames(p, fields, k, 1, dropouts=drops, overcorrect=oc, intra=intra, threads=8)
        frames.append(out[0])
        stats.append(tuple(st))
    return np.stack(frames), stats


@pytest.mark.parametrize("fmt", ["yuv444p16", "yuv444ps"])
def test_pal2d_kind(cuda, tmp_path, fmt):
    cap = capture(NF, 41)
    path = _write(tmp_path, cap)
    got, _, _, _ = _decode_all(path, abi.DEC_PAL_2D, fmt, chroma_gain=1.1)
    ref, _ = O.decode_frames(O.params(1, FMTS[fmt], chroma_gain=1.1), cap.fields, 0, NF // 2, threads=8)
    _compare(got, ref, fmt)
    # AUTO resolves to CHD_DEC_PAL_2D for a PAL source (registry.cpp:96-107)
    auto, _, _, _ = _decode_all(path, abi.DEC_AUTO, fmt, chroma_gain=1.1)
    assert np.array_equal(auto, got)


@pytest.mark.parametrize("kind,okind,fmt,level", [(abi.DEC_TRANSFORM_3D, 3, "yuv444p16", 1.5),
                                                  (abi.DEC_TRANSFORM_2D, 2, "yuv444ps", 4.0),
                                                  (abi.DEC_PAL_2D, 1, "yuv444ps", 2.5)])
def test_luma_noise_coring(cuda, tmp_path, kind, okind, fmt, level):
    cap = capture(NF, 42)
    path = _write(tmp_path, cap)
    got, _, _, _ = _decode_all(path, kind, fmt, luma_nr_level=level)
    ref, _ = O.decode_frames(O.params(okind, FMTS[fmt], y_nr_level=level), cap.fields, 0, NF // 2, threads=8)
    _compare(got, ref, fmt)


@pytest.mark.parametrize("fmt,clamp,cdp,bsp,pad", [("rgb48", "none", "modern", "scientific", 1),
                                                   ("rgbs", "legal_ycbcr_bt601", "classic", "modern", 1),
                                                   ("rgbs", "legal_rgb_hdr", "modern", "classic", 1),
                                                   ("gray16", "legal_rgb_sdr", "modern", "scientific", 16),
                                                   ("grays", "legal_ycbcr_bt601", "modern", "scientific", 1),
                                                   ("yuv444p16", "none", "classic", "classic", 1)])
def test_output_formats(cuda, tmp_path, fmt, clamp, cdp, bsp, pad):
    cap = capture(NF, 43)
    path = _write(tmp_path, cap)
    got, _, d, _ = _decode_all(path, abi.DEC_TRANSFORM_3D, fmt, output_clamp=clamp, color_difference_precision=cdp,
                               broadcast_scaling_precision=bsp, padding_multiple=pad)
    clamps = {"none": 0, "legal_rgb_sdr": 1, "legal_rgb_hdr": 2, "legal_ycbcr_bt601": 3}
    p = O.params(3, FMTS[fmt], clamp_mode=clamps[clamp], padding_multiple=pad)
    O.colour_precision(p, cdp, bsp)
    ref, _ = O.decode_frames(p, cap.fields, 0, NF // 2, threads=8)
    oi = d.output_info()
    assert oi.num_planes == (1 if fmt.startswith("gray") else 3)
    _compare(got, ref, fmt)


def test_reverse_field_order(cuda, tmp_path):
    """reverse_field_order pairs each first field with the second field before
    it (LdDecodeMetaData::getFieldNumber, src/metadata/core.cpp:1117-1179):
    frame k = capture fields (2k+2, 2k+1), first field still in slot 0."""
    cap = capture(NF, 44, dropouts=0.02)
    path = _write(tmp_path, cap)
    got, stats, d, _ = _decode_all(path, abi.DEC_TRANSFORM_3D, reverse_field_order=True, dropout=(False, False))
    n = NF // 2 - 1
    assert d.output_info().num_frames == n
    order = [i for k in range(n) for i in (2 * k + 2, 2 * k + 1)]
    arr = np.ascontiguousarray(cap.fields[order])
    pos = {src: j for j, src in enumerate(order)}
    drops = [(pos[f], s[0], s[1], s[2]) for f, spans in enumerate(cap.dropouts) for s in spans if f in pos]
    ref, rstats = _oracle_frames(O.params(3, O.FMT_P16), arr, n, drops)
    _compare(got, ref, "yuv444p16")
    assert stats == rstats
    p = O.params(3, O.FMT_P16)
    for k in range(n):
        assert sorted(d.dropout_spans(k)) == sorted(O.dropout_spans(p, drops, k, 0))


def test_subcarrier_locked_capture(cuda, tmp_path):
    """isSubcarrierLocked PAL: every window frame's second field is shifted 2
    samples left with 2 black samples appended, its dropouts moved with it
    (SourceField::shiftSecondField, src/decoders/source_field.cpp:45-66)."""
    cap = capture(NF, 45, dropouts=0.02)
    path = _write(tmp_path, cap, sc_locked=True)
    got, stats, d, v = _decode_all(path, abi.DEC_TRANSFORM_3D, dropout=(True, False))
    assert v.info().is_subcarrier_locked == 1
    drops = O.flatten_dropouts(cap.dropouts)
    p = O.params(3, O.FMT_P16, sc_locked=1)
    ref, rstats = _oracle_frames(p, cap.fields, NF // 2, drops, oc=True)
    _compare(got, ref, "yuv444p16")
    assert stats == rstats
    for k in range(NF // 2):
        for mode in (0, 1):
            assert sorted(d.dropout_spans(k, mode)) == sorted(O.dropout_spans(p, drops, k, mode))


@pytest.mark.parametrize("kind,okind", [(8, 3), (7, 2)])
def test_device_field_parity_swap(cuda, kind, okind):
    """chdg first_field_offset = 1: even-indexed fields are second fields
    (the golden 'rev' cases of the reference harness)."""
    torch = cuda
    from libchromadec_gb300 import device as D
    cap = capture(NF + 1, 46)
    fields = np.ascontiguousarray(cap.fields[1:])
    n = NF // 2
    eng = D.Engine(D.default_geometry(), D.default_config(kind=kind, fmt=D.FMT_P16, first_field_offset=1))
    dfields = torch.from_numpy(fields.reshape(NF, -1).view(np.int16)).cuda()
    out = torch.empty((n, 3, 576, 948), dtype=torch.int16, device="cuda")
    eng.decode(dfields, 0, n, out)
    torch.cuda.synchronize()
    ref, _ = O.decode_frames(O.params(okind, O.FMT_P16, first_field_offset=1), fields, 0, n, threads=8)
    _compare(out.cpu().numpy().view(np.uint16), ref, "yuv444p16")
