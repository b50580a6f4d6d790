"""Seeded synthetic captures shared by the tests (cached per process)."""
import functools

import numpy as np

from libchromadec_gb300 import synth


@functools.lru_cache(maxsize=8)
def capture(nfields: int, seed: int, pan_x: float = 1.5, pan_y: float = 0.5, dropouts: float = 0.0):
    cfg = synth.SynthConfig(seed=seed, pan_x=pan_x, pan_y=pan_y, dropout_line_fraction=dropouts)
    return synth.make_capture(nfields, cfg)
