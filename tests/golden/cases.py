"""Cases of the golden vectors (tests/golden/golden.json).

Each case names the reference code path (decode / chroma-only / dropout
concealment), the Transform-PAL kind (2 or 3), the output format, the frames
decoded and the options. Inputs are seeded synthetic PAL captures from
libchromadec_gb300.synth; frames at both ends of a capture exercise the black
padding of the 3D field window.
"""
from __future__ import annotations

import functools

import numpy as np

from libchromadec_gb300 import synth

CASES = {
    "t2d_p16": dict(mode="decode", kind=2, fmt="p16", nfields=8, seed=31, first=0, count=4),
    "t2d_ps": dict(mode="decode", kind=2, fmt="ps", nfields=8, seed=31, first=0, count=4),
    "t2d_thr": dict(mode="decode", kind=2, fmt="p16", nfields=8, seed=31, first=1, count=2, thr_seed=5),
    "t2d_opts_ps": dict(mode="decode", kind=2, fmt="ps", nfields=8, seed=31, first=2, count=2, threshold=0.55,
                        chroma_gain=0.8, chroma_phase_deg=-12.0, clamp_mode=1),
    "t3d_p16": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=0, count=6),
    "t3d_ps": dict(mode="decode", kind=3, fmt="ps", nfields=12, seed=32, first=0, count=6),
    "t3d_thr": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=2, count=2, thr_seed=6),
    "t3d_opts": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=32, first=0, count=3, chroma_gain=1.25,
                     chroma_phase_deg=7.5, clamp_mode=3, padding_multiple=32, active_start=185, active_end=1101,
                     first_active_frame_line=50, last_active_frame_line=601),
    "t3d_drop": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02),
    "t3d_drop_oc": dict(mode="decode", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02,
                        overcorrect=1),
    "t3d_drop_intra": dict(mode="decode", kind=3, fmt="ps", nfields=12, seed=33, first=1, count=4, dropouts=0.02,
                           intra=1),
    "conceal": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02),
    "conceal_oc": dict(mode="dropout", kind=3, fmt="p16", nfields=12, seed=33, first=0, count=6, dropouts=0.02,
                       overcorrect=1),
    "chroma2d": dict(mode="chroma", kind=2, nfields=8, seed=31, first=0, count=4),
    "chroma3d": dict(mode="chroma", kind=3, nfields=12, seed=32, first=0, count=6),
}


@functools.lru_cache(maxsize=8)
def _capture(nfields: int, seed: int, dropouts: float):
    cfg = synth.SynthConfig(seed=seed, pan_x=1.5, pan_y=0.5, dropout_line_fraction=dropouts)
    return synth.make_capture(nfields, cfg)


def case_inputs(case: dict):
    """(fields uint16 (n, 313, 1135), flat dropouts [(field, startx, endx, fieldLine)] or None)."""
    cap = _capture(case["nfields"], case["seed"], case.get("dropouts", 0.0))
    flat = None
    if case.get("dropouts", 0.0) > 0:
        flat = [(f, s[0], s[1], s[2]) for f, spans in enumerate(cap.dropouts) for s in spans]
    return np.ascontiguousarray(cap.fields), flat


def thresholds_for(case: dict):
    if "thr_seed" not in case:
        return None
    n = 80 if case["kind"] == 2 else 768
    return np.random.default_rng(case["thr_seed"]).uniform(0.25, 0.65, n)
