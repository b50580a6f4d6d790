"""Precision report of the tensor-core form (chdg_tc3d_spectra).

The tensor-core form computes the Transform-PAL 3D tile spectra with split
TF32 or BF16 products; this module holds what the report compares them with:
the same spectra in FP64 (numpy's FFT over the reference's tile,
TransformPal3D::forwardFFTTile, src/decoders/palcolour/transform_pal_3d.cpp:
168-202) and the threshold decision of every visited bin
(TransformPal3D::applyFilter, transform_pal_3d.cpp:249-333). It is
measurement code for the tests and the benchmark: the decoder never calls it.
"""
from __future__ import annotations

import numpy as np

KQ_KX = 5      # kx = 2..6
KY = 32
KZ = 8


def tile_grid(geometry):
    """(tileX0, tileY0, ntx, nty) of the 3D tiles (transform_pal_3d.cpp:123-165)."""
    tx0 = geometry.active_start - 8
    ntx = (geometry.active_end - tx0 + 7) // 8
    ty0 = geometry.first_active_frame_line - 16
    nty = (geometry.last_active_frame_line - ty0) // 16 + 1
    return tx0, ty0, ntx, nty


def _window(n):
    return 0.5 - 0.5 * np.cos(2.0 * np.pi * (np.arange(n) + 0.5) / n)


def fp64_spectra(fields: np.ndarray, m: int, tiles, geometry, swap: int = 0) -> np.ndarray:
    """FP64 spectra of Z tile m (fields 2m .. 2m+7) at the given spatial tiles:
    complex128 [len(tiles), 8 kz, 5 kx (2..6), 32 ky]. fields: uint16
    (nfields, field_height, field_width)."""
    tiles = np.asarray(tiles, dtype=np.int64)
    nf, fh, fw = fields.shape
    flat = fields.reshape(nf, fh * fw).astype(np.float64) - geometry.black
    tx0, ty0, ntx, nty = tile_grid(geometry)
    fafl, lafl = geometry.first_active_frame_line, geometry.last_active_frame_line
    T = np.zeros((len(tiles), 8, 32, 16))
    tileX = tx0 + 8 * (tiles % ntx)
    tileY = ty0 + 16 * (tiles // ntx)
    x = np.arange(16)
    for z in range(8):
        f = 2 * m + z
        if f < 0 or f >= nf:
            continue
        p = (f & 1) ^ swap
        for y in range(32):
            L = tileY + y
            ok = ((L & 1) == p) & (L >= fafl) & (L <= lafl)
            if not ok.any():
                continue
            idx = (L[:, None] >> 1) * fw + tileX[:, None] + x[None, :]
            idx = np.clip(idx, 0, fh * fw - 1)
            T[ok, z, y, :] = flat[f][idx[ok]]
    w = _window(8)[:, None, None] * _window(32)[None, :, None] * _window(16)[None, None, :]
    S = np.fft.rfftn(T * w[None], axes=(1, 2, 3))          # [t, kz, ky, 9]
    return np.ascontiguousarray(S[:, :, :, 2:7].transpose(0, 1, 3, 2))


def keep_mask(S: np.ndarray, threshold: float, dtype=np.float64) -> np.ndarray:
    """Chroma (keep) decision of every visited bin (kx = 2..4) of spectra S
    [..., 8 kz, 5 kx, 32 ky]: kept when |bin|^2 and |mirror|^2 are within
    threshold^2 of each other (the mirror about the carrier is
    ((10 - kz) & 7, 8 - kx, (40 - ky) & 31)); the carrier, its own mirror, is
    always kept. The magnitudes and comparisons run in `dtype`."""
    mag = (S.real.astype(dtype) ** 2 + S.imag.astype(dtype) ** 2).astype(dtype)
    t2 = dtype(threshold) * dtype(threshold)
    kz = np.arange(8)
    ky = np.arange(32)
    kzr = (10 - kz) & 7
    kyr = (40 - ky) & 31
    out = np.zeros(S.shape[:-3] + (8, 3, 32), dtype=bool)
    for k in range(3):          # kx = 2 + k, mirror kx = 6 - k (index 4 - k)
        a = mag[..., :, k, :]
        b = mag[..., kzr, 4 - k, :][..., :, kyr]
        sim = (a - b * t2 >= 0) & (b - a * t2 >= 0)
        if k == 2:
            self_bin = (kz[:, None] == kzr[:, None]) & (ky[None, :] == kyr[None, :])
            sim = sim | self_bin
        out[..., :, k, :] = sim
    return out


def report(S_tc: np.ndarray, S_ref: np.ndarray, threshold: float) -> dict:
    """Errors of the tensor-core spectra against FP64 and the decisions that flip."""
    d = S_tc.astype(np.complex128) - S_ref
    err = np.abs(d)
    scale = np.sqrt(np.mean(np.abs(S_ref) ** 2))
    keep_tc = keep_mask(S_tc, threshold, np.float32)
    keep_ref = keep_mask(S_ref, threshold, np.float64)
    return {
        "max_abs_err": float(err.max()),
        "rms_err": float(np.sqrt(np.mean(err ** 2))),
        "rms_rel_err": float(np.sqrt(np.mean(err ** 2)) / scale) if scale > 0 else 0.0,
        "max_rel_err": float(err.max() / np.abs(S_ref).max()) if np.abs(S_ref).max() > 0 else 0.0,
        "bins": int(keep_ref.size),
        "flips": int(np.count_nonzero(keep_tc != keep_ref)),
        "flip_fraction": float(np.count_nonzero(keep_tc != keep_ref) / keep_ref.size),
    }
