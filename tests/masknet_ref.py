"""FP64 restatement of the learned chroma-mask network (test infrastructure).

The checker for the library's mask-network kernels (csrc/masknet.cu): the
forward pass, the loss and every parameter gradient, in float64 numpy, with
the bf16 roundings at the points the GPU rounds (features, weights, each
layer's post-ReLU activations, and the back-propagated pre-activation
gradients that feed the next contraction), so that the GPU's FP32
accumulation is the only difference. The reference library has no such
network for PAL; its NTSC nnTransform3D decoder is the precedent for a
learned per-bin mask on a 3D tile spectrum
(src/decoders/nntransform3d/nntransform3d_pipeline_cuda.cu:160-244).

Tile domain (one 8 x 32 x 16 Transform-PAL 3D tile's spectrum, the bins the
filter can keep): kz 0..7 and ky 0..31 (both periodic), q = kx - 2 in 0..4
(zero beyond). A voxel is v = (q * 8 + kz) * 32 + ky. Input channels: the
bin's feature f = ln(1 + |X|) / 16 and the feature of its mirror about the
carrier, (kz, ky, kx) -> ((10 - kz) mod 8, (40 - ky) mod 32, 8 - kx)
(TransformPal3D::applyFilter, src/decoders/palcolour/transform_pal_3d.cpp:
280-300). Three 3x3x3 convolutions of 16 channels with ReLU, then a 1x1x1
sigmoid head: p, the fraction of each bin kept as chroma.

Parameters (flat float32 vector, this order): W1[27][2][16], b1[16],
W2[27][16][16], b2[16], W3[27][16][16], b3[16], wh[16], bh; tap
t = (dz + 1) * 9 + (dy + 1) * 3 + (dq + 1).

Loss of a batch: L = sum |p X - C|^2 / sum |X|^2 with C the true chroma
spectrum; per bin the data are a = |X|^2 and c = Re(C conj X), so
dL/dp = 2 (p a - c) / S.
"""
from __future__ import annotations

import numpy as np

NQ, NZ, NY, NC, NCIN = 5, 8, 32, 16, 2
NV = NQ * NZ * NY
SIZES = [("W1", 27 * NCIN * NC), ("b1", NC), ("W2", 27 * NC * NC), ("b2", NC), ("W3", 27 * NC * NC),
         ("b3", NC), ("wh", NC), ("bh", 1)]
NPARAM = sum(n for _, n in SIZES)
FEATURE_SCALE = 1.0 / 16.0


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return (u.astype(np.uint32)).view(np.float32).astype(np.float64)


def split(params: np.ndarray) -> dict:
    out, o = {}, 0
    for name, n in SIZES:
        out[name] = np.asarray(params[o:o + n], dtype=np.float64)
        o += n
    out["W1"] = out["W1"].reshape(27, NCIN, NC)
    out["W2"] = out["W2"].reshape(27, NC, NC)
    out["W3"] = out["W3"].reshape(27, NC, NC)
    return out


def join(g: dict) -> np.ndarray:
    return np.concatenate([np.asarray(g[name], dtype=np.float64).reshape(-1) for name, _ in SIZES])


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation; the head starts at p = 1/2 everywhere."""
    rng = np.random.default_rng(seed)
    p = {}
    p["W1"] = rng.standard_normal((27, NCIN, NC)) * np.sqrt(2.0 / (27 * NCIN))
    p["b1"] = np.zeros(NC)
    p["W2"] = rng.standard_normal((27, NC, NC)) * np.sqrt(2.0 / (27 * NC))
    p["b2"] = np.zeros(NC)
    p["W3"] = rng.standard_normal((27, NC, NC)) * np.sqrt(2.0 / (27 * NC))
    p["b3"] = np.zeros(NC)
    p["wh"] = rng.standard_normal(NC) * np.sqrt(1.0 / NC)
    p["bh"] = np.zeros(1)
    return join(p).astype(np.float32)


def _taps():
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dq in (-1, 0, 1):
                yield (dz + 1) * 9 + (dy + 1) * 3 + (dq + 1), dz, dy, dq


def _shift(x: np.ndarray, dz: int, dy: int, dq: int) -> np.ndarray:
    """y[..., q, z, y] = x[..., q + dq, (z + dz) mod 8, (y + dy) mod 32], zero outside q."""
    s = np.roll(np.roll(x, -dz, axis=-2), -dy, axis=-1)
    out = np.zeros_like(s)
    if dq == 0:
        out[:] = s
    elif dq > 0:
        out[..., :-dq, :, :] = s[..., dq:, :, :]
    else:
        out[..., -dq:, :, :] = s[..., :dq, :, :]
    return out


def conv(x: np.ndarray, W: np.ndarray) -> np.ndarray:
    """x (B, Ci, 5, 8, 32), W (27, Ci, Co) -> (B, Co, 5, 8, 32)."""
    out = 0.0
    for t, dz, dy, dq in _taps():
        out = out + np.einsum("bcqzy,cd->bdqzy", _shift(x, dz, dy, dq), W[t])
    return out


def conv_t(g: np.ndarray, W: np.ndarray) -> np.ndarray:
    """Gradient of conv with respect to its input: (B, Co, ...) -> (B, Ci, ...)."""
    out = 0.0
    for t, dz, dy, dq in _taps():
        out = out + _shift(np.einsum("bdqzy,cd->bcqzy", g, W[t]), -dz, -dy, -dq)
    return out


def conv_w(x: np.ndarray, g: np.ndarray) -> np.ndarray:
    """Gradient of conv with respect to W: x (B, Ci, ...), g (B, Co, ...) -> (27, Ci, Co)."""
    out = np.zeros((27, x.shape[1], g.shape[1]))
    for t, dz, dy, dq in _taps():
        out[t] = np.einsum("bcqzy,bdqzy->cd", _shift(x, dz, dy, dq), g)
    return out


def mirror(f: np.ndarray) -> np.ndarray:
    """f[..., q, z, y] -> f[..., 4 - q, (10 - z) mod 8, (40 - y) mod 32]."""
    q = 4 - np.arange(NQ)
    z = (10 - np.arange(NZ)) % NZ
    y = (40 - np.arange(NY)) % NY
    return f[..., q[:, None, None], z[None, :, None], y[None, None, :]]


def features(X: np.ndarray) -> np.ndarray:
    """bf16 feature of each bin: ln(1 + |X|) / 16."""
    return bf16(np.log1p(np.abs(X)) * FEATURE_SCALE)


def forward(params: np.ndarray, feat: np.ndarray, rounding: bool = True):
    """feat (B, 5, 8, 32) -> p (B, 5, 8, 32) and the activations."""
    r = bf16 if rounding else (lambda a: np.asarray(a, dtype=np.float64))
    P = split(params)
    W1, W2, W3, wh = r(P["W1"]), r(P["W2"]), r(P["W3"]), r(P["wh"])
    f = r(feat)
    x0 = np.stack([f, mirror(f)], axis=1)
    a1 = r(np.maximum(conv(x0, W1) + P["b1"][None, :, None, None, None], 0.0))
    a2 = r(np.maximum(conv(a1, W2) + P["b2"][None, :, None, None, None], 0.0))
    a3 = r(np.maximum(conv(a2, W3) + P["b3"][None, :, None, None, None], 0.0))
    z = np.einsum("bcqzy,c->bqzy", a3, wh) + P["bh"][0]
    p = 1.0 / (1.0 + np.exp(-z))
    return p, dict(x0=x0, a1=a1, a2=a2, a3=a3, W1=W1, W2=W2, W3=W3, wh=wh)


def loss_and_grad(params: np.ndarray, feat: np.ndarray, a: np.ndarray, c: np.ndarray, rounding: bool = True):
    """Loss (without the constant sum |C|^2 term) and the gradient of every
    parameter. a = |X|^2, c = Re(C conj X), shapes (B, 5, 8, 32)."""
    r = bf16 if rounding else (lambda v: np.asarray(v, dtype=np.float64))
    p, A = forward(params, feat, rounding)
    S = float(np.sum(a))
    L = float(np.sum(p * p * a - 2.0 * p * c)) / S
    dp = 2.0 * (p * a - c) / S
    dz = dp * p * (1.0 - p)
    g = {}
    g["bh"] = np.array([dz.sum()])
    g["wh"] = np.einsum("bqzy,bcqzy->c", dz, A["a3"])
    dz3 = r(dz[:, None] * A["wh"][None, :, None, None, None] * (A["a3"] > 0))
    g["b3"] = dz3.sum(axis=(0, 2, 3, 4))
    g["W3"] = conv_w(A["a2"], dz3)
    dz2 = r(conv_t(dz3, A["W3"]) * (A["a2"] > 0))
    g["b2"] = dz2.sum(axis=(0, 2, 3, 4))
    g["W2"] = conv_w(A["a1"], dz2)
    dz1 = r(conv_t(dz2, A["W2"]) * (A["a1"] > 0))
    g["b1"] = dz1.sum(axis=(0, 2, 3, 4))
    g["W1"] = conv_w(A["x0"], dz1)
    return L, join(g), p


def fallback(p: np.ndarray, limit: float = 0.1) -> np.ndarray:
    """Tiles whose mean |p - 1/2| is below `limit` fall back to the threshold."""
    return np.mean(np.abs(p - 0.5), axis=(1, 2, 3)) < limit
