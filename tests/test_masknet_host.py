"""The learned-mask network's FP64 restatement (tests/masknet_ref.py), on
the CPU: its gradients against central finite differences, the mirror map,
and the parameter layout the library's header declares."""
import os
import re

import numpy as np

from tests import masknet_ref as R

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parameter_count_matches_header():
    h = open(os.path.join(ROOT, "include", "chromadec_gb300.h")).read()
    assert int(re.search(r"#define CHDG_MASKNET_PARAMS (\d+)", h).group(1)) == R.NPARAM == 14753
    assert int(re.search(r"#define CHDG_MASKNET_BINS (\d+)", h).group(1)) == R.NV


def test_mirror_is_the_filter_reflection_and_an_involution():
    f = np.random.default_rng(0).standard_normal((R.NQ, R.NZ, R.NY))
    assert np.array_equal(R.mirror(R.mirror(f)), f)
    # bin (kz, ky, kx) -> ((10 - kz) % 8, (40 - ky) % 32, 8 - kx), transform_pal_3d.cpp:280-300
    m = R.mirror(f)
    for q, z, y in ((0, 0, 0), (1, 3, 7), (2, 5, 4), (4, 7, 31)):
        assert m[q, z, y] == f[4 - q, (10 - z) % 8, (40 - y) % 32]


def _problem(seed, b=2):
    rng = np.random.default_rng(seed)
    params = R.init_params(seed).astype(np.float64)
    params[-1] = 0.3                                   # a head bias away from 0
    feat = rng.uniform(0.0, 1.0, (b, R.NQ, R.NZ, R.NY))
    a = rng.uniform(0.1, 2.0, feat.shape)
    c = a * rng.uniform(-0.2, 1.2, feat.shape)
    return params, feat, a, c


def test_gradients_match_finite_differences():
    params, feat, a, c = _problem(1)
    L, g, _ = R.loss_and_grad(params, feat, a, c, rounding=False)
    rng = np.random.default_rng(2)
    offsets, o = {}, 0
    for name, n in R.SIZES:
        offsets[name] = (o, n)
        o += n
    eps = 1e-6
    for name, (o, n) in offsets.items():
        for i in rng.choice(n, size=min(n, 6), replace=False):
            k = o + int(i)
            pp, pm = params.copy(), params.copy()
            pp[k] += eps
            pm[k] -= eps
            fd = (R.loss_and_grad(pp, feat, a, c, rounding=False)[0] -
                  R.loss_and_grad(pm, feat, a, c, rounding=False)[0]) / (2 * eps)
            assert abs(fd - g[k]) <= 1e-5 * max(1e-3, abs(fd), abs(g[k])), (name, i, fd, g[k])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 3.0e38], dtype=np.float32)
    got = R.bf16(x)
    assert got[0] == 1.0 and got[1] == 1.0 and got[2] == 1.0 + 2 ** -6 and got[3] == -2.5
