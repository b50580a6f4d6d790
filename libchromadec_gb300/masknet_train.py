"""Training of the learned chroma mask (chdg_masknet_*) on the GPU.

Pairs come from the pipeline itself: seeded synthetic component video (luma
zone plates, blurred random U/V patches, high-saturation edges, colour bars;
pans of 0-4 px/field, AWGN sigma 0-2 % of white - black) is PAL-encoded by
synth.py; the feature pass of the learned walk (chdg_learned_features) gives
every Z tile's features and spectrum X of the composite, and the same pass
over the encoder's chroma-only signal gives the true chroma spectrum C. The
network's loss is sum |p X - C|^2 / sum |X|^2; each step is one batch of
tiles through the library's forward, backward and Adam kernels.

    python -m libchromadec_gb300.masknet_train --steps 20000 --out weights.f32

Device buffers are torch tensors (allocation, gathering a batch's tiles);
every forward, backward and optimiser step runs in libchromadec_gb300.so.
"""
from __future__ import annotations

import argparse
import json
import os
import time
from dataclasses import dataclass

import numpy as np

from . import device as D
from . import synth

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_WEIGHTS = os.path.join(HERE, "data", "tpal3d_masknet.f32")
CHROMA_OFFSET = 32768      # the chroma-only signal is stored as offset + C


def load_weights(path: str = DEFAULT_WEIGHTS) -> np.ndarray:
    w = np.fromfile(path, dtype="<f4")
    if w.size != D.MASKNET_PARAMS:
        raise ValueError(f"{path}: {w.size} parameters, expected {D.MASKNET_PARAMS}")
    return w


def save_weights(w: np.ndarray, path: str) -> None:
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    np.ascontiguousarray(w, dtype="<f4").tofile(path)


def training_config(rng: np.random.Generator, seed: int) -> synth.SynthConfig:
    return synth.SynthConfig(seed=seed, pan_x=float(rng.uniform(0.0, 4.0)), pan_y=float(rng.uniform(0.0, 1.0)),
                             noise=float(rng.uniform(0.0, 0.02)), bars=bool(rng.random() < 0.5),
                             zone_plate=True, patches=True, patch_amplitude=float(rng.uniform(0.15, 0.45)),
                             patch_sigma=float(rng.uniform(8.0, 30.0)),
                             saturation_edges=bool(rng.random() < 0.6))


def init_weights(seed: int) -> np.ndarray:
    """He-style initialisation of the convolutions (zero biases); the head
    starts with small weights, so every fraction starts near 1/2."""
    rng = np.random.default_rng(seed)
    parts = [rng.standard_normal(27 * 2 * 16) * np.sqrt(2.0 / 54), np.zeros(16),
             rng.standard_normal(27 * 16 * 16) * np.sqrt(2.0 / 432), np.zeros(16),
             rng.standard_normal(27 * 16 * 16) * np.sqrt(2.0 / 432), np.zeros(16),
             rng.standard_normal(16) * 0.05, np.zeros(1)]
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == D.MASKNET_PARAMS
    return w


def chroma_only_fields(cap: synth.SynthCapture) -> np.ndarray:
    return np.clip(np.rint(CHROMA_OFFSET + cap.chroma), 0, 65535).astype(np.uint16)


def luma_only_fields(cap: synth.SynthCapture) -> np.ndarray:
    return np.clip(np.rint(synth.BLACK + (synth.WHITE - synth.BLACK) * cap.y), 0, 65535).astype(np.uint16)


@dataclass
class TileSet:
    feat: object      # int16 CUDA tensor (ntiles, 1280): bf16 bits
    ac: object        # float32 CUDA tensor (ntiles, 1280, 2)
    energy: object    # float32 CUDA tensor (ntiles,): sum |X|^2


def capture_pairs(cap: synth.SynthCapture, stream=None) -> TileSet:
    """Every Z tile of a capture's frames: features and (|X|^2, Re(C conj X))."""
    import torch
    n = cap.fields.shape[0]
    nfr = n // 2
    g = D.default_geometry()
    eng = D.Engine(g, D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
    gc = D.default_geometry()
    gc.black = CHROMA_OFFSET
    engc = D.Engine(gc, D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
    nt = eng.ntiles()
    nz = nfr + 2
    comp = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    chro = torch.from_numpy(chroma_only_fields(cap).reshape(n, -1).view(np.int16)).cuda()
    feat = torch.empty((nz * nt, D.MASKNET_BINS), dtype=torch.int16, device="cuda")
    sx = torch.empty((nz * nt, D.MASKNET_BINS, 2), dtype=torch.float32, device="cuda")
    sc = torch.empty_like(sx)
    scratch = torch.empty((nz * nt, D.MASKNET_BINS), dtype=torch.int16, device="cuda")
    eng.learned_features(comp, 0, nfr, feat, sx, None, stream)
    engc.learned_features(chro, 0, nfr, scratch, sc, None, stream)
    ac = torch.empty_like(sx)
    D.masknet_pairs(sx, sc, nz * nt * D.MASKNET_BINS, ac, stream)
    torch.cuda.synchronize()
    energy = ac[..., 0].sum(dim=1)
    eng.close()
    engc.close()
    return TileSet(feat=feat, ac=ac, energy=energy)


def build_training_set(n_captures: int, nfields: int, seed: int, min_energy_frac: float = 1e-3, log=print):
    """Tiles of n_captures seeded captures, keeping those with more than
    min_energy_frac of the median tile energy (flat picture areas carry no
    signal for the loss)."""
    import torch
    rng = np.random.default_rng(seed)
    feats, acs = [], []
    t0 = time.time()
    for k in range(n_captures):
        cfg = training_config(rng, seed + 1 + k)
        cap = synth.make_capture(nfields, cfg, truth=True)
        ts = capture_pairs(cap)
        thr = float(ts.energy.median()) * min_energy_frac
        keep = torch.nonzero(ts.energy > thr).squeeze(1)
        feats.append(ts.feat.index_select(0, keep))
        acs.append(ts.ac.index_select(0, keep))
        del ts
        log(f"capture {k + 1}/{n_captures}: pan ({cfg.pan_x:.2f}, {cfg.pan_y:.2f}) noise {cfg.noise:.4f} "
            f"edges {cfg.saturation_edges}: {keep.numel()} tiles ({time.time() - t0:.0f} s)")
    return TileSet(feat=torch.cat(feats), ac=torch.cat(acs), energy=None)


def train(steps: int = 20000, batch: int = 256, lr: float = 1e-3, lr_end: float = 2e-5, seed: int = 1000,
          n_captures: int = 16, nfields: int = 24, init=None, log=print):
    """Train from `init` (default: a seeded He initialisation); returns the
    weights and a record of the run."""
    import torch
    data = build_training_set(n_captures, nfields, seed, log=log)
    ntiles = data.feat.shape[0]
    w0 = init_weights(seed) if init is None else np.asarray(init, dtype=np.float32)
    net = D.MaskNet(w0)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    # a fixed evaluation batch for the loss curve
    ev = torch.randint(0, ntiles, (4 * batch,), device="cuda", generator=gen)
    evf, eva = data.feat.index_select(0, ev).contiguous(), data.ac.index_select(0, ev).contiguous()
    curve = []
    loss0, _ = net.train_step(evf, eva, evf.shape[0], 0.0)
    curve.append((0, loss0))
    log(f"{ntiles} training tiles; step 0 loss {loss0:.5f}")
    t0 = time.time()
    for s in range(1, steps + 1):
        idx = torch.randint(0, ntiles, (batch,), device="cuda", generator=gen)
        f = data.feat.index_select(0, idx)
        a = data.ac.index_select(0, idx)
        frac = (s - 1) / max(1, steps - 1)
        step_lr = lr_end + 0.5 * (lr - lr_end) * (1.0 + np.cos(np.pi * frac))
        net.train_step(f, a, batch, float(step_lr), want_loss=False)
        if s % max(1, steps // 20) == 0 or s == steps:
            l, _ = net.train_step(evf, eva, evf.shape[0], 0.0)
            curve.append((s, l))
            log(f"step {s}: loss {l:.5f} ({time.time() - t0:.0f} s)")
    w = net.weights()
    rec = {"steps": steps, "batch": batch, "lr": lr, "lr_end": lr_end, "seed": seed, "n_captures": n_captures,
           "fields_per_capture": nfields, "training_tiles": ntiles, "loss_curve": curve,
           "train_seconds": time.time() - t0}
    net.close()
    return w, rec


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1000)
    ap.add_argument("--captures", type=int, default=16)
    ap.add_argument("--fields", type=int, default=24)
    ap.add_argument("--out", default=DEFAULT_WEIGHTS)
    ap.add_argument("--record", default=None, help="write the run's record (loss curve) as JSON here")
    a = ap.parse_args()
    w, rec = train(a.steps, a.batch, a.lr, seed=a.seed, n_captures=a.captures, nfields=a.fields)
    save_weights(w, a.out)
    if a.record:
        with open(a.record, "w") as fp:
            json.dump(rec, fp, indent=1)
    print(json.dumps({k: v for k, v in rec.items() if k != "loss_curve"}))


if __name__ == "__main__":
    main()
