"""GPU parity through the reference-compatible chd_* ABI.

A seeded synthetic capture is written as an ld-decode .tbc + JSON sidecar,
opened with chd_video_open_composite and decoded with chd_decode_frame /
chd_decode_frames_async exactly as a consumer of the reference would; every
frame is compared with the CPU oracle on the same fields. Tolerances as in
the device-level tests: yuv444p16 within +-1 LSB everywhere, yuv444ps within
1e-4; dropout statistics, spans and masks bit-exact.
"""
import numpy as np
import pytest

from libchromadec_gb300 import abi, synth
from oracle import oracle as O
from tests._capture import capture

pytestmark = pytest.mark.gpu

NF = 16   # fields -> 8 frames


@pytest.fixture(scope="module")
def tbc(tmp_path_factory):
    cap = capture(NF, 21, dropouts=0.01)
    path = str(tmp_path_factory.mktemp("abi") / "cap.tbc")
    synth.write_tbc(path, cap)
    return path, cap


def _compare(got, ref, fmt):
    if fmt == "yuv444ps":
        err = np.abs(got.astype(np.float64) - ref.astype(np.float64)).max()
        assert err < 1e-4, err
    else:
        d = np.abs(got.astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 1, (d.max(), (d > 0).mean())


def _decoder(path, kind=abi.DEC_TRANSFORM_3D, fmt="yuv444p16", **opts):
    v = abi.Video(path)
    d = abi.Decoder(v, kind)
    d.set("output_format", fmt)
    for k, val in opts.items():
        d.set(k, val)
    d.commit()
    return v, d


@pytest.mark.parametrize("fmt", ["yuv444p16", "yuv444ps"])
def test_sequential_decode_matches_oracle(cuda, tbc, fmt):
    path, cap = tbc
    v, d = _decoder(path, fmt=fmt)
    oi = d.output_info()
    assert (oi.width, oi.height, oi.num_planes, oi.num_frames) == (948, 576, 3, NF // 2)
    assert oi.format == (abi.PIXEL_YUV444PS if fmt == "yuv444ps" else abi.PIXEL_YUV444P16)
    ref, _ = O.decode_frames(O.params(3, O.FMT_PS if fmt == "yuv444ps" else O.FMT_P16), cap.fields, 0, NF // 2,
                             threads=8)
    for k in range(NF // 2):
        f = d.decode(k)
        assert f.index == k and (f.info.width, f.info.height) == (948, 576)
        _compare(f.planes(), ref[k], fmt)
        f.close()


def test_random_access_and_reuse(cuda, tbc):
    path, cap = tbc
    v, d = _decoder(path)
    ref, _ = O.decode_frames(O.params(3, O.FMT_P16), cap.fields, 0, NF // 2, threads=8)
    frames = [d.decode(k) for k in (5, 2, 3, 4, 7, 0)]
    for f in frames:        # all alive at once: chunks are shared, not reused
        _compare(f.planes(), ref[f.index], "yuv444p16")
    for f in frames:
        f.close()
    f = d.decode(1)
    _compare(f.planes(), ref[1], "yuv444p16")
    with pytest.raises(abi.ChdError) as e:
        d.decode(NF // 2)
    assert e.value.status == abi.E_OUT_OF_RANGE


def test_dropout_correction_matches_oracle(cuda, tbc):
    path, cap = tbc
    v, d = _decoder(path)
    flat = O.flatten_dropouts(cap.dropouts)
    assert len(flat) > 0
    for overcorrect, intra in ((False, False), (True, False), (False, True)):
        d.set_dropout(True, overcorrect, intra)
        for k in range(NF // 2):
            ref, st = O.decode_frames(O.params(3, O.FMT_P16), cap.fields, k, 1, dropouts=flat,
                                      overcorrect=overcorrect, intra=intra, threads=8)
            f = d.decode(k)
            _compare(f.planes(), ref[0], "yuv444p16")
            assert d.last_dropout_stats() == tuple(st), (k, overcorrect, intra)
            f.close()
    d.set_dropout(False)
    ref, _ = O.decode_frames(O.params(3, O.FMT_P16), cap.fields, 3, 1, threads=8)
    f = d.decode(3)
    _compare(f.planes(), ref[0], "yuv444p16")
    assert d.last_dropout_stats() == (0, 0, 0)


def test_concealed_fields_match_oracle_byte_for_byte(cuda, tbc):
    """The composite the transform reads after the GPU concealment kernel,
    compared sample for sample with the oracle's DropoutCorrector
    (src/dropout/dropout_corrector.cpp:50-157, 469-530): every mode, every
    frame, every sample of both fields."""
    path, cap = tbc
    v, d = _decoder(path)
    flat = O.flatten_dropouts(cap.dropouts)
    p = O.params(3, O.FMT_P16)
    changed = 0
    for overcorrect, intra in ((False, False), (True, False), (False, True)):
        d.set_dropout(True, overcorrect, intra)
        for k in range(NF // 2):
            got = d.concealed_fields(k)
            ref, st = O.dropout_correct_frame(p, cap.fields, k, flat, overcorrect=overcorrect, intra=intra)
            assert got.dtype == np.uint16 and got.shape == ref.shape
            bad = np.argwhere(got != ref)
            assert bad.size == 0, (k, overcorrect, intra, bad[:5])
            changed += int((got != cap.fields[2 * k:2 * k + 2]).sum())
    assert changed > 0                                    # the kernel did conceal something
    d.set_dropout(False)
    assert np.array_equal(d.concealed_fields(2), cap.fields[4:6])


def test_async_delivery_cancel_and_errors(cuda, tbc):
    path, cap = tbc
    v, d = _decoder(path)
    ref, _ = O.decode_frames(O.params(3, O.FMT_P16), cap.fields, 0, NF // 2, threads=8)
    res = d.decode_async([3, 0, 1, 1, 99, 7, -1, 2])
    assert len(res) == 8
    bad = sorted(i for s, i, _ in res if s == abi.E_OUT_OF_RANGE)
    assert bad == [-1, 99]
    good = [(i, p) for s, i, p in res if s == abi.OK]
    assert sorted(i for i, _ in good) == [0, 1, 1, 2, 3, 7]
    for i, p in good:
        _compare(p, ref[i], "yuv444p16")
    # cancellation requested from inside a callback: the rest report CHD_E_CANCELLED
    res = d.decode_async(list(range(NF // 2)), cancel_after=1)
    assert len(res) == NF // 2
    st = [s for s, _, _ in res]
    assert st[0] == abi.OK and abi.E_CANCELLED in st
    assert all(s in (abi.OK, abi.E_CANCELLED) for s in st)
    assert sorted(i for _, i, _ in res) == list(range(NF // 2))


def test_dropout_mask_on_gpu_matches_spans(cuda, tbc):
    path, cap = tbc
    for fmt, dtype, on in (("yuv444p16", np.uint16, 0xFFFF), ("yuv444ps", np.float32, 1.0)):
        v, d = _decoder(path, fmt=fmt)
        for k in range(NF // 2):
            for mode in (abi.DROPOUT_DETECTED, abi.DROPOUT_OVERCORRECT):
                m = d.dropout_mask(k, mode)
                want = np.zeros((576, 948), dtype=dtype)
                for y, x0, x1, _ in d.dropout_spans(k, mode):
                    want[y, x0:x1] = on
                assert m.dtype == dtype and np.array_equal(m, want)


@pytest.mark.parametrize("fmt", ["yuv444p16", "yuv444ps"])
def test_transform2d_through_abi(cuda, tbc, fmt):
    path, cap = tbc
    v, d = _decoder(path, kind=abi.DEC_TRANSFORM_2D, fmt=fmt, transform_threshold=0.5)
    p = O.params(2, O.FMT_PS if fmt == "yuv444ps" else O.FMT_P16, threshold=0.5)
    ref, _ = O.decode_frames(p, cap.fields, 0, NF // 2, threads=8)
    res = d.decode_async(list(range(NF // 2)))
    assert [s for s, _, _ in res] == [abi.OK] * (NF // 2)
    for _, i, planes in res:
        _compare(planes, ref[i], fmt)


def test_padding_crop_gain_phase_through_abi(cuda, tbc):
    path, cap = tbc
    v, d = _decoder(path, padding_multiple=32, first_active_sample=185, last_active_sample=1100,
                    first_active_frame_line=50, last_active_frame_line=601, chroma_gain=1.25,
                    chroma_phase_deg=7.5, output_clamp="legal_ycbcr_bt601")
    p = O.params(3, O.FMT_P16, chroma_gain=1.25, chroma_phase_deg=7.5, clamp_mode=3, padding_multiple=32)
    p.active_start, p.active_end = 185, 1101
    p.first_active_frame_line, p.last_active_frame_line = 50, 601
    w, h, _, _ = O.output_geometry(p)
    oi = d.output_info()
    assert (oi.width, oi.height) == (w, h) and w % 32 == 0 and h % 32 == 0
    ref, _ = O.decode_frames(p, cap.fields, 0, NF // 2, threads=8)
    for k in (0, 1, 6, 7):
        f = d.decode(k)
        _compare(f.planes(), ref[k], "yuv444p16")


def test_thresholds_file_through_abi(cuda, tbc, tmp_path):
    path, cap = tbc
    rng = np.random.default_rng(4)
    thr = rng.uniform(0.25, 0.65, 768)
    f = tmp_path / "thr3d.txt"
    f.write_text("\n".join(repr(float(t)) for t in thr))
    v, d = _decoder(path, transform_thresholds_file=str(f))
    ref, _ = O.decode_frames(O.params(3, O.FMT_P16, thresholds=list(thr)), cap.fields, 0, NF // 2, threads=8)
    for k in range(NF // 2):
        fr = d.decode(k)
        _compare(fr.planes(), ref[k], "yuv444p16")


def test_truncated_capture_decodes_missing_frames_as_black(cuda, tmp_path):
    """A .tbc shorter than its sidecar: frames whose fields are missing enter
    the window as black fields (SourceField::loadFields' blank fallback,
    src/decoders/source_field.cpp:110-158), uploaded by the device fill."""
    cap = capture(NF, 23)
    path = str(tmp_path / "short.tbc")
    synth.write_tbc(path, cap)
    with open(path, "r+b") as fp:
        fp.truncate(13 * cap.fields[0].nbytes)       # fields 14..16 (1-based) missing
    black = cap.fields.copy()
    black[12:] = synth.BLACK                          # frames 6 and 7 become blank
    ref, _ = O.decode_frames(O.params(3, O.FMT_P16), black, 0, NF // 2, threads=8)
    v, d = _decoder(path)
    res = d.decode_async(list(range(NF // 2)))
    assert [s for s, _, _ in res] == [abi.OK] * (NF // 2)
    for _, i, planes in res:
        _compare(planes, ref[i], "yuv444p16")
