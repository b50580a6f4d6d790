"""Tensor-core form of the Transform-PAL 3D forward transform on the GPU.

chdg_tc3d_spectra (tcgen05 split-precision contractions) against the FP64
spectra of the same tiles: 3xTF32 within 2e-5 of the spectrum's RMS per bin
(RMS error), BF16x3 within 2e-3; the threshold decisions taken on the
tensor-core spectra agree with the FP64 ones on all but a small fraction of
bins; Z tiles wholly in the black padding are exactly zero."""
import numpy as np
import pytest

from libchromadec_gb300 import device as D
from libchromadec_gb300 import tc_study as T
from tests._capture import capture

pytestmark = pytest.mark.gpu

NF = 24


@pytest.fixture(scope="module")
def spectra(cuda):
    torch = cuda
    cap = capture(NF, seed=11)
    g = D.default_geometry()
    tx0, ty0, ntx, nty = T.tile_grid(g)
    ntiles = ntx * nty
    fields = torch.from_numpy(cap.fields.reshape(NF, -1).view(np.int16)).cuda()
    m_begin, m_end = -5, 10   # -5: all-black window; -2..-1: partly padding; 8, 9: past the end
    out = {}
    for variant in (D.TC_3XTF32, D.TC_BF16X3):
        spec = torch.full((m_end - m_begin, ntiles, 8, 5, 32), float("nan"), dtype=torch.complex64, device="cuda")
        D.tc3d_spectra(fields, m_begin, m_end, spec, variant)
        D.tc3d_sync()
        out[variant] = spec.cpu().numpy()
    return cap, g, ntiles, m_begin, m_end, out


@pytest.mark.parametrize("variant,rms_tol,max_tol", [(D.TC_3XTF32, 2e-5, 2e-4), (D.TC_BF16X3, 2e-3, 2e-2)])
def test_tc_spectra_match_fp64(spectra, variant, rms_tol, max_tol):
    cap, g, ntiles, m_begin, m_end, out = spectra
    S = out[variant]
    assert np.isfinite(S).all()
    rng = np.random.default_rng(7)
    tiles = np.unique(np.concatenate([rng.choice(ntiles, 150, replace=False), [0, 119, ntiles - 120, ntiles - 1]]))
    flips = bins = 0
    worst = {"rms_rel_err": 0.0, "max_rel_err": 0.0}
    for m in range(m_begin + 1, m_end):
        ref = T.fp64_spectra(cap.fields, m, tiles, g)
        r = T.report(S[m - m_begin][tiles], ref, 0.4)
        worst = {k: max(worst[k], r[k]) for k in worst}
        flips += r["flips"]
        bins += r["bins"]
    print(f"variant {variant}: {worst}, flips {flips} of {bins}")
    assert worst["rms_rel_err"] < rms_tol
    assert worst["max_rel_err"] < max_tol
    assert flips / bins < (1e-3 if variant == D.TC_3XTF32 else 2e-2)


def test_tc_black_window_is_zero(spectra):
    cap, g, ntiles, m_begin, m_end, out = spectra
    for variant in out:
        assert np.all(out[variant][0] == 0)   # Z tile -5: fields -10 .. -3
