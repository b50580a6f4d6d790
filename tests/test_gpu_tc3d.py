"""Tensor-core form of the Transform-PAL 3D forward transform on the GPU.

chdg_tc3d_spectra (tcgen05 split-precision contractions) against the FP64
spectra of the same tiles: 3xTF32 within 2e-5 of the spectrum's RMS per bin
(RMS error), BF16x3 within 2e-3; the threshold decisions taken on the
tensor-core spectra agree with the FP64 ones on all but a small fraction of
bins; Z tiles wholly in the black padding are exactly zero."""
import numpy as np
import pytest

from libchromadec_gb300 import device as D
from tests import tc_study as T
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


def _psnr(x, ref, peak):
    mse = float(np.mean((x.astype(np.float64) - ref) ** 2))
    return 10.0 * np.log10(peak * peak / mse)


@pytest.fixture(scope="module")
def decoded(cuda):
    """The 16-field capture decoded by the plain form and both tensor-core
    variants: chroma planes and yuv444ps frames, with the FP64 oracle's and
    the encoder's ground truth."""
    torch = cuda
    from libchromadec_gb300 import synth
    from oracle import oracle as O
    cfg = synth.SynthConfig(seed=13, pan_x=1.5, pan_y=0.5)
    cap = synth.make_capture(16, cfg, truth=True)
    fields = torch.from_numpy(cap.fields.reshape(16, -1).view(np.int16)).cuda()
    res = {}
    for form in (-1, D.TC_3XTF32, D.TC_BF16X3):
        eng = D.Engine(D.default_geometry(), D.default_config(kind=8, fmt=D.FMT_PS))
        eng.set_tc_form(form)
        chroma = torch.empty((16, 288, 948), dtype=torch.float32, device="cuda")
        eng.chroma(fields, 0, 8, chroma)
        frames = torch.empty((8, 3, eng.out_height, eng.out_width), dtype=torch.float32, device="cuda")
        eng.decode(fields, 0, 8, frames)
        torch.cuda.synchronize()
        D.tc3d_sync()
        res[form] = (chroma.cpu().numpy(), frames.cpu().numpy())
    ref_frames, _ = O.decode_frames(O.params(3, O.FMT_PS), cap.fields, 0, 8, threads=8)
    truth = cap.chroma[:, 22:310, 177:1125]
    return cap, res, ref_frames, truth


@pytest.mark.parametrize("form,rms_tol,max_tol", [(D.TC_3XTF32, 2e-5, 2e-2), (D.TC_BF16X3, 2e-4, 5e-2)])
def test_tc_decode_error_per_plane(decoded, form, rms_tol, max_tol):
    """yuv444ps of the tensor-core form against the FP64 oracle, per plane;
    the plain form is within the parity tolerance everywhere."""
    cap, res, ref, truth = decoded
    plain = res[-1][1]
    assert np.abs(plain - ref).max() <= 1e-4
    got = res[form][1]
    assert np.isfinite(got).all()
    for pl, name in enumerate("Y Cb Cr".split()):
        d = np.abs(got[:, pl] - ref[:, pl])
        print(f"form {form} {name}: max {d.max():.3e} rms {np.sqrt(np.mean(d * d)):.3e}")
        assert np.sqrt(np.mean(d * d)) < rms_tol
        assert d.max() < max_tol


def test_tc_chroma_psnr_matches_plain(decoded):
    """Chroma separated by each form against the encoder's true chroma: the
    tensor-core forms reach the plain form's PSNR (within 0.05 dB)."""
    cap, res, ref, truth = decoded
    peak = 54016.0 - 16384.0
    ps = {form: _psnr(res[form][0][4:12], truth[4:12], peak) for form in res}
    print("chroma PSNR dB:", ps)
    assert ps[-1] > 25.0
    for form in (D.TC_3XTF32, D.TC_BF16X3):
        assert abs(ps[form] - ps[-1]) < 0.05


def test_tc_form_through_host_buffers(cuda):
    """The tensor-core form through chdg_decode_host (double-buffered field
    windows that start mid-capture) equals its device-resident decode."""
    import ctypes as C
    torch = cuda
    cap = capture(NF, seed=17)
    eng = D.Engine(D.default_geometry(), D.default_config(kind=8, fmt=D.FMT_P16))
    eng.set_tc_form(D.TC_3XTF32)
    nfr = NF // 2
    dev_fields = torch.from_numpy(cap.fields.reshape(NF, -1).view(np.int16)).cuda()
    dev_out = torch.empty((nfr, 3, eng.out_height, eng.out_width), dtype=torch.int16, device="cuda")
    eng.decode(dev_fields, 0, nfr, dev_out)
    host_fields = torch.from_numpy(cap.fields.reshape(NF, -1).view(np.int16)).pin_memory()
    host_out = torch.empty((nfr, 3, eng.out_height, eng.out_width), dtype=torch.int16).pin_memory()
    rc = D.lib().chdg_decode_host(eng._h, C.c_void_p(host_fields.data_ptr()), host_fields[0].numel(), NF, 0, nfr,
                                  C.c_void_p(host_out.data_ptr()), None)
    assert rc == 0
    torch.cuda.synchronize()
    D.tc3d_sync()
    assert np.array_equal(host_out.numpy(), dev_out.cpu().numpy())
