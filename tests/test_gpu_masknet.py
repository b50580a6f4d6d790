"""GPU tests of the learned form's kernels (csrc/masknet.cu, the learned
walk passes of csrc/tpal3d.cu) against the FP64 restatement
(tests/masknet_ref.py) and the FP64 tile spectra: the network's forward
pass, the gradient of every layer, the feature pass, and the apply pass fed
with the threshold decisions."""
import numpy as np
import pytest

from tests import masknet_ref as R
from tests import tc_study as T
from tests._capture import capture

pytestmark = pytest.mark.gpu


def _bf16_bits(x):
    import torch
    return torch.from_numpy(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).view(torch.int16)


def _problem(seed, b):
    rng = np.random.default_rng(seed)
    params = R.init_params(seed)
    params[-1] = 0.2
    feat = R.bf16(rng.uniform(0.0, 1.0, (b, R.NQ, R.NZ, R.NY)))
    a = rng.uniform(0.1, 2.0, feat.shape)
    c = a * rng.uniform(-0.2, 1.2, feat.shape)
    return params, feat, a, c


@pytest.mark.parametrize("tensor_cores,b", [(True, 6), (False, 6), (True, 153)])
def test_forward_matches_restatement(cuda, tensor_cores, b):
    """b = 153 with one CTA per SM: one CTA runs two tiles (the next tile's
    input written during the first one's head), the others one."""
    torch = cuda
    from libchromadec_gb300 import device as D
    params, feat, _, _ = _problem(3, b)
    net = D.MaskNet(params)
    net.set_tensor_cores(tensor_cores)
    f = _bf16_bits(feat.reshape(b, -1)).cuda()
    p = torch.empty((b, R.NV), dtype=torch.float32, device="cuda")
    fb = torch.empty(b, dtype=torch.uint8, device="cuda")
    net.forward(f, b, p, fb)
    net.sync()
    ref, _ = R.forward(params.astype(np.float64), feat)
    got = p.cpu().numpy().reshape(ref.shape)
    assert np.abs(got - ref).max() < 3e-3, np.abs(got - ref).max()
    conf = np.mean(np.abs(ref - 0.5), axis=(1, 2, 3))
    want = conf < 0.1
    sure = np.abs(conf - 0.1) > 1e-3
    assert np.array_equal(fb.cpu().numpy().astype(bool)[sure], want[sure])
    net.close()


@pytest.mark.parametrize("tensor_cores", [True, False])
def test_gradient_of_every_layer_matches_restatement(cuda, tensor_cores):
    torch = cuda
    from libchromadec_gb300 import device as D
    b = 5
    params, feat, a, c = _problem(4, b)
    net = D.MaskNet(params)
    net.set_tensor_cores(tensor_cores)
    f = _bf16_bits(feat.reshape(b, -1)).cuda()
    ac = torch.from_numpy(np.stack([a, c], axis=-1).reshape(b, R.NV, 2).astype(np.float32)).cuda()
    loss, grad = net.train_step(f, ac, b, 0.0, want_loss=True, want_grad=True)
    L, gref, _ = R.loss_and_grad(params.astype(np.float64), feat, a, c)
    assert abs(loss - L) <= 1e-4 * abs(L), (loss, L)
    o = 0
    for name, n in R.SIZES:
        g, r = grad[o:o + n].astype(np.float64), gref[o:o + n]
        err = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-30)
        assert err < 1e-2, (name, err)
        o += n
    # an Adam step moves the weights and lowers the loss on the same batch
    net.train_step(f, ac, b, 1e-3, want_loss=False)
    l2, _ = net.train_step(f, ac, b, 0.0)
    assert l2 < loss
    net.close()


def test_feature_pass_matches_fp64_tile_spectra(cuda):
    torch = cuda
    from libchromadec_gb300 import device as D
    cap = capture(16, 61)
    fields = torch.from_numpy(cap.fields.reshape(16, -1).view(np.int16)).cuda()
    eng = D.Engine(D.default_geometry(), D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
    nt = eng.ntiles()
    fb, fe = 2, 5
    nz = fe - fb + 2
    feat = torch.empty((nz, nt, R.NV), dtype=torch.int16, device="cuda")
    spec = torch.empty((nz, nt, R.NV, 2), dtype=torch.float32, device="cuda")
    thr = torch.empty((nz, nt, R.NV), dtype=torch.float32, device="cuda")
    eng.learned_features(fields, fb, fe, feat, spec, thr)
    torch.cuda.synchronize()
    featf = feat.view(torch.bfloat16).float().cpu().numpy()
    S = spec.cpu().numpy()
    S = S[..., 0] + 1j * S[..., 1]
    keep = thr.cpu().numpy()
    g = D.default_geometry()
    tiles = np.random.default_rng(0).choice(nt, 200, replace=False)
    for zi in range(nz):
        m = fb - 2 + zi
        ref = T.fp64_spectra(cap.fields, m, tiles, g)             # [t, kz, q, ky]
        # the walk's horizontal origin is the tile centre (x = 7.5): its
        # spectrum is the reference's times exp(i pi kx 15 / 16)
        ref = ref * np.exp(1j * np.pi * (2 + np.arange(5)) * 15.0 / 16.0)[None, None, :, None]
        ref = ref.transpose(0, 2, 1, 3).reshape(len(tiles), R.NV)   # v = (q * 8 + kz) * 32 + ky
        got = S[zi, tiles]
        scale = np.abs(ref).max()
        assert np.abs(got - ref).max() <= 2e-6 * scale + 1e-3
        fref = np.log1p(np.abs(ref)) / 16.0
        assert np.abs(featf[zi, tiles] - fref).max() <= 2 ** -7 * 1.1
        # threshold decisions of the visited bins and their mirrors, away from the boundary
        km = T.keep_mask(T.fp64_spectra(cap.fields, m, tiles, g), 0.4)   # [t, kz, 3, ky]
        kv = keep[zi, tiles].reshape(len(tiles), 5, 8, 32)
        agree = (kv[:, :3].transpose(0, 2, 1, 3) > 0.5) == km
        assert agree.mean() > 0.9999, agree.mean()


def test_apply_pass_with_threshold_decisions(cuda):
    """The apply pass fed with the feature pass's threshold decisions gives
    the same chroma whether they come as fractions 0/1 or as fallback flags,
    and that chroma is the plain form's wherever FP32 decided as exactly."""
    torch = cuda
    from libchromadec_gb300 import device as D
    cap = capture(20, 62)
    n = 20
    fields = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    eng = D.Engine(D.default_geometry(), D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
    nt = eng.ntiles()
    fb, fe = 1, 9
    nz = fe - fb + 2
    feat = torch.empty((nz, nt, R.NV), dtype=torch.int16, device="cuda")
    thr = torch.empty((nz, nt, R.NV), dtype=torch.float32, device="cuda")
    eng.learned_features(fields, fb, fe, feat, None, thr)
    zero = torch.zeros((nz, nt), dtype=torch.uint8, device="cuda")
    ones = torch.ones((nz, nt), dtype=torch.uint8, device="cuda")
    a = torch.empty((2 * (fe - fb), 288, 948), dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    plain = torch.empty_like(a)
    eng.learned_chroma(fields, fb, fe, thr, zero, a)
    eng.learned_chroma(fields, fb, fe, torch.zeros_like(thr), ones, b)
    eng.chroma(fields, fb, fe, plain)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    # FP32 decisions equal the exact ones except on the guard-band bins the
    # plain form corrected; each such flip changes one tile's output (at most
    # 4 fields x 16 rows x 16 samples)
    _, flips = eng.stats()
    off = int(((a - plain).abs() > 2e-2).sum())
    assert off <= 1024 * flips, (off, flips)


def test_short_training_lowers_the_loss(cuda):
    """A few hundred steps of the library's own training kernels on pairs the
    encoder generates lower the loss on a fixed batch."""
    from libchromadec_gb300 import masknet_train as MT
    w, rec = MT.train(steps=300, batch=64, lr=2e-3, seed=5000, n_captures=2, nfields=12, log=lambda *a: None)
    curve = rec["loss_curve"]
    assert np.all(np.isfinite(w))
    assert curve[-1][1] < curve[0][1] - 0.1 * abs(curve[0][1]), curve


def test_trained_network_beats_the_threshold_on_held_out_fields(cuda):
    """The committed network (trained on seeds >= 1001) against the plain
    0.4 threshold on a held-out capture: at least 1 dB higher chroma PSNR
    against the encoder's chroma, and less cross-colour energy (it lets a
    little more chroma stay in the luma -- cross-luma -- than the threshold
    does, for far less luma detail taken as chroma)."""
    from libchromadec_gb300 import masknet_train as MT
    from tests import learned_eval as E
    res = E.evaluate(MT.load_weights(), nfields=60, seed=1, chunk_frames=30)
    pl, le = res["plain"], res["learned"]
    assert le["chroma_psnr_db"] > pl["chroma_psnr_db"] + 1.0, res
    assert le["cross_colour_rel_energy"] < 0.5 * pl["cross_colour_rel_energy"], res
    assert le["cross_colour_rel_energy"] + le["cross_luma_rel_energy"] < \
        pl["cross_colour_rel_energy"] + pl["cross_luma_rel_energy"], res


def test_tensor_core_and_cuda_core_forward_agree_on_trained_weights(cuda):
    """The trained network over real tile features: both forward kernels give
    the same fractions up to FP32 accumulation order (and the rare bf16
    activation that rounds the other way)."""
    torch = cuda
    from libchromadec_gb300 import device as D, masknet_train as MT
    cap = capture(16, 63)
    fields = torch.from_numpy(cap.fields.reshape(16, -1).view(np.int16)).cuda()
    eng = D.Engine(D.default_geometry(), D.default_config(kind=D.KIND_TRANSFORM_3D))
    nt = eng.ntiles()
    feat = torch.empty((5 * nt, R.NV), dtype=torch.int16, device="cuda")
    eng.learned_features(fields, 2, 5, feat)
    net = D.MaskNet(MT.load_weights())
    out = []
    for tc in (True, False):
        net.set_tensor_cores(tc)
        p = torch.empty((5 * nt, R.NV), dtype=torch.float32, device="cuda")
        fb = torch.empty(5 * nt, dtype=torch.uint8, device="cuda")
        net.forward(feat, 5 * nt, p, fb)
        net.sync()
        out.append((p, fb))
    d = (out[0][0] - out[1][0]).abs()
    assert float(d.max()) < 2e-2 and float(d.mean()) < 1e-5
    assert float((out[0][1] != out[1][1]).float().mean()) < 1e-3


def test_learned_decode_is_independent_of_the_batch_split(cuda):
    """An engine limited to 64-frame batches decodes 72 frames as a 64-frame
    batch and an 8-frame one, and each batch's edge Z tiles read fields
    outside it: frames 56-71 come out bit for bit as a decode of those 16
    frames in one batch, and as the same engine's default 256-frame batch;
    and the learned engine's chroma equals the feature pass, network and
    apply pass run one by one."""
    torch = cuda
    from libchromadec_gb300 import device as D, masknet_train as MT
    n = 144
    cap = capture(n, 64)
    fields = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    net = D.MaskNet(MT.load_weights())
    eng = D.Engine(D.default_geometry(), D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
    eng.set_masknet(net)
    whole = torch.empty((72, 3, 576, 948), dtype=torch.float32, device="cuda")
    one = torch.empty_like(whole)
    part = torch.empty((16, 3, 576, 948), dtype=torch.float32, device="cuda")
    eng.decode(fields, 0, 72, one)
    eng.set_max_batch_frames(64)
    eng.decode(fields, 0, 72, whole)
    eng.decode(fields, 56, 72, part)
    torch.cuda.synchronize()
    assert torch.isfinite(whole).all()
    assert torch.equal(whole, one)
    assert torch.equal(whole[56:72], part)
    with pytest.raises(RuntimeError):
        eng.set_max_batch_frames(0)

    fb, fe = 60, 68
    nz = fe - fb + 2
    direct = torch.empty((2 * (fe - fb), 288, 948), dtype=torch.float32, device="cuda")
    eng.chroma(fields, fb, fe, direct)
    plain = D.Engine(D.default_geometry(), D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_PS))
    nt = plain.ntiles()
    feat = torch.empty((nz * nt, R.NV), dtype=torch.int16, device="cuda")
    plain.learned_features(fields, fb, fe, feat)
    p = torch.empty((nz * nt, R.NV), dtype=torch.float32, device="cuda")
    fbk = torch.empty(nz * nt, dtype=torch.uint8, device="cuda")
    net.forward(feat, nz * nt, p, fbk)
    manual = torch.empty_like(direct)
    plain.learned_chroma(fields, fb, fe, p, fbk, manual)
    torch.cuda.synchronize()
    assert torch.equal(direct, manual)
    eng.set_masknet(None)
    net.close()
