"""Host side of the tensor-core form (no GPU): the coefficient operand images
the library builds for tcgen05 (split hi/lo, K-major no-swizzle core-matrix
layout) decode to the windowed DFT matrices of the X, Y and Z stages, and the
FP64 reference and decision rule of the precision report follow the
reference's tile and filter."""
import numpy as np
import pytest

from libchromadec_gb300 import device as D
from tests import tc_study as T


def _rc(n):
    return 0.5 - 0.5 * np.cos(2.0 * np.pi * (np.arange(n) + 0.5) / n)


def _decode(img: bytes, rows: int, K: int, variant: int) -> np.ndarray:
    """Inverse of the shared-memory layout: element (r, k) at
    (r / 8) * 8 * row_bytes + (k * eb / 16) * 128 + (r % 8) * 16 + (k * eb) % 16."""
    eb = 4 if variant == 0 else 2
    rb = K * eb
    raw = np.frombuffer(img, dtype=np.uint8)
    out = np.zeros((rows, K))
    for r in range(rows):
        for k in range(K):
            o = (r >> 3) * 8 * rb + ((k * eb) >> 4) * 128 + (r & 7) * 16 + ((k * eb) & 15)
            if variant == 0:
                out[r, k] = raw[o:o + 4].view(np.float32)[0]
            else:
                out[r, k] = (raw[o:o + 2].view(np.uint16).astype(np.uint32) << 16).view(np.float32)[0]
    return out


def _expected(stage: int, y0: int) -> np.ndarray:
    if stage == 0:
        M = np.zeros((16, 16))
        x = np.arange(16)
        for k in range(5):
            th = 2 * np.pi * (k + 2) * x / 16
            M[2 * k] = _rc(16) * np.cos(th)
            M[2 * k + 1] = -_rc(16) * np.sin(th)
        return M
    if stage == 1:
        M = np.zeros((64, 32))
        y = y0 + 2 * np.arange(16)
        w = _rc(32)[y]
        for ky in range(32):
            ph = 2 * np.pi * ky * y / 32
            M[2 * ky, :16] = w * np.cos(ph)
            M[2 * ky, 16:] = w * np.sin(ph)
            M[2 * ky + 1, :16] = -w * np.sin(ph)
            M[2 * ky + 1, 16:] = w * np.cos(ph)
        return M
    M = np.zeros((16, 16))
    z = np.arange(8)
    for kz in range(8):
        ph = 2 * np.pi * kz * z / 8
        M[2 * kz, :8] = _rc(8) * np.cos(ph)
        M[2 * kz, 8:] = _rc(8) * np.sin(ph)
        M[2 * kz + 1, :8] = -_rc(8) * np.sin(ph)
        M[2 * kz + 1, 8:] = _rc(8) * np.cos(ph)
    return M


@pytest.mark.parametrize("variant", [D.TC_3XTF32, D.TC_BF16X3])
@pytest.mark.parametrize("stage,y0", [(0, 0), (1, 0), (1, 1), (2, 0)])
def test_operand_images_decode_to_the_dft_matrices(variant, stage, y0):
    rows, K = {0: (16, 16), 1: (64, 32), 2: (16, 16)}[stage]
    hi = _decode(D.tc3d_operand(variant, stage, y0, 0), rows, K, variant)
    lo = _decode(D.tc3d_operand(variant, stage, y0, 1), rows, K, variant)
    M = _expected(stage, y0)
    # hi alone is the input type's rounding; hi + lo carries twice its bits
    hi_bits, pair_tol = (11, 2.0 ** -21) if variant == D.TC_3XTF32 else (8, 2.0 ** -15)
    assert np.max(np.abs(hi - M)) <= 2.0 ** -hi_bits
    assert np.max(np.abs(hi + lo - M)) <= pair_tol
    if variant == D.TC_3XTF32:   # TF32: the low 13 bits of every word are zero
        raw = np.frombuffer(D.tc3d_operand(variant, stage, y0, 0), dtype=np.uint32)
        assert not np.any(raw & 0x1FFF)


def test_fp64_spectra_follow_the_reference_tile():
    """One tile by a direct triple DFT sum: own-parity rows from the field,
    the rest black, windowed, bins kx = 2..6."""
    g = D.default_geometry()
    rng = np.random.default_rng(3)
    fields = rng.integers(0x1000, 0xE000, size=(12, g.field_height, g.field_width)).astype(np.uint16)
    tx0, ty0, ntx, nty = T.tile_grid(g)
    assert (tx0, ty0, ntx, nty) == (169, 28, 120, 37)
    tile, m = 3 * ntx + 17, 1
    S = T.fp64_spectra(fields, m, [tile], g)[0]
    tileX, tileY = tx0 + 8 * (tile % ntx), ty0 + 16 * (tile // ntx)
    t = np.zeros((8, 32, 16))
    for z in range(8):
        f = 2 * m + z
        for y in range(32):
            L = tileY + y
            if (L & 1) == (f & 1) and g.first_active_frame_line <= L <= g.last_active_frame_line:
                row = fields[f].reshape(-1)[(L >> 1) * g.field_width + tileX:(L >> 1) * g.field_width + tileX + 16]
                t[z, y] = row.astype(np.float64) - g.black
    w = _rc(8)[:, None, None] * _rc(32)[None, :, None] * _rc(16)[None, None, :]
    tw = t * w
    zz, yy, xx = np.meshgrid(np.arange(8), np.arange(32), np.arange(16), indexing="ij")
    for kz, ky, kx in [(0, 0, 2), (3, 20, 4), (7, 31, 6), (5, 9, 3)]:
        direct = np.sum(tw * np.exp(-2j * np.pi * (kz * zz / 8 + ky * yy / 32 + kx * xx / 16)))
        assert abs(S[kz, kx - 2, ky] - direct) <= 1e-9 * max(1.0, abs(direct))


def test_keep_mask_is_the_mirror_threshold_rule():
    rng = np.random.default_rng(9)
    S = rng.normal(size=(8, 5, 32)) + 1j * rng.normal(size=(8, 5, 32))
    keep = T.keep_mask(S, 0.4)
    for kz in range(8):
        for k in range(3):
            for ky in range(32):
                kzr, kyr = (10 - kz) & 7, (40 - ky) & 31
                a = abs(S[kz, k, ky]) ** 2
                b = abs(S[kzr, 4 - k, kyr]) ** 2
                want = (a - b * 0.16 >= 0) and (b - a * 0.16 >= 0)
                if k == 2 and kz == kzr and ky == kyr:
                    want = True
                assert keep[kz, k, ky] == want
    r = T.report(S.astype(np.complex64), S, 0.4)
    assert r["bins"] == 768 and r["flips"] == 0 and r["max_rel_err"] < 1e-6


def test_tc_entry_points_reject_bad_arguments():
    """chdg_tc3d_* and chdg_engine_set_tc_form validate before any CUDA call."""
    import ctypes as C
    L = D.lib()
    g = D.default_geometry()
    buf = (C.c_uint8 * 16)()
    # spectra: bad variant, empty Z range, null buffers, a stride shorter than a field
    assert L.chdg_tc3d_spectra(C.byref(g), 2, C.c_void_p(16), 355255, 8, 0, 1, C.c_void_p(16), None) == -1
    assert L.chdg_tc3d_spectra(C.byref(g), 0, C.c_void_p(16), 355255, 8, 3, 3, C.c_void_p(16), None) == -1
    assert L.chdg_tc3d_spectra(C.byref(g), 0, None, 355255, 8, 0, 1, C.c_void_p(16), None) == -1
    assert L.chdg_tc3d_spectra(C.byref(g), 0, C.c_void_p(16), 1000, 8, 0, 1, C.c_void_p(16), None) == -1
    assert b"bad argument" in L.chd_last_error()
    # operand images: stage, split and buffer size
    assert L.chdg_tc3d_operand(0, 6, 0, 0, buf, 16) == -1
    assert L.chdg_tc3d_operand(0, 0, 0, 2, buf, 16) == -1
    assert L.chdg_tc3d_operand(0, 0, 0, 0, buf, 16) == -1   # 2 KB image, 16-byte buffer
    assert b"too small" in L.chd_last_error()
    assert L.chdg_engine_set_tc_form(None, 0) == -1


def test_tc_operand_sizes():
    """Image sizes: rows x K x element bytes (TF32 4, BF16 2)."""
    for variant, eb in ((D.TC_3XTF32, 4), (D.TC_BF16X3, 2)):
        for stage, (rows, K) in enumerate([(16, 16), (64, 32), (16, 16), (16, 16), (32, 64), (16, 16)]):
            assert len(D.tc3d_operand(variant, stage, 0, 0)) == rows * K * eb


def test_report_counts_flips():
    """A bin pushed across the threshold is one flip per visited bin it decides."""
    rng = np.random.default_rng(4)
    S = rng.normal(size=(8, 5, 32)) + 1j * rng.normal(size=(8, 5, 32))
    # bin (kz 1, kx 2, ky 3) and its mirror (kz 1, kx 6, ky 5): equal magnitudes, then one scaled
    S[1, 0, 3] = 1.0
    S[1, 4, 5] = 1.0
    T_ = S.copy()
    T_[1, 0, 3] = 10.0   # |a|^2 = 100 against 1: dissimilar at t = 0.4
    r = T.report(T_.astype(np.complex64), S, 0.4)
    assert r["flips"] == 1 and r["bins"] == 768
