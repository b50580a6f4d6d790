"""GPU parity of the Transform-PAL 3D path against the CPU oracle.

The oracle (oracle/tpal_oracle.c) is the C restatement of the reference's
TransformPal3D / PALcolour / OutputWriter, bit-identical to the reference's
own sources built against the same FP64 DFT. Tolerances: chroma within
2e-2 sample units (FP32 arithmetic; every threshold decision must match,
a flipped decision shows up as an error of tens to hundreds of units),
yuv444ps within 1e-4 absolute, yuv444p16 within +-1 LSB everywhere.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests._capture import capture

pytestmark = pytest.mark.gpu


def _engine(kind=8, fmt=0, **kw):
    from libchromadec_gb300 import device as D
    return D.Engine(D.default_geometry(), D.default_config(kind=kind, fmt=fmt, **kw))


def test_chroma_matches_oracle(cuda):
    torch = cuda
    cap = capture(16, seed=5)
    fields = torch.from_numpy(cap.fields.reshape(16, -1).view(np.int16)).cuda()
    eng = _engine()
    nfr = 8
    out = torch.empty((2 * nfr, 288, 948), dtype=torch.float32, device="cuda")
    eng.chroma(fields, 0, nfr, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref = O.transform_chroma(O.params(kind=3), cap.fields, 0, nfr)[:, 22:310, 177:1125]
    err = np.abs(got - ref)
    exact, flips = eng.stats()
    print("max chroma err", err.max(), "exact decisions", exact, "fp32 flips", flips)
    assert err.max() < 2e-2


@pytest.mark.parametrize("fmt", [0, 1])
def test_decode_matches_oracle(cuda, fmt):
    torch = cuda
    cap = capture(16, seed=5)
    fields = torch.from_numpy(cap.fields.reshape(16, -1).view(np.int16)).cuda()
    eng = _engine(fmt=fmt)
    nfr = 8
    dt = torch.float32 if fmt == 1 else torch.int16
    out = torch.empty((nfr, 3, 576, 948), dtype=dt, device="cuda")
    eng.decode(fields, 0, nfr, out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    ref, _ = O.decode_frames(O.params(kind=3, fmt=fmt), cap.fields, 0, nfr, threads=8)
    if fmt == 1:
        err = np.abs(got - ref)
        print("ps max err", err.max())
        assert err.max() < 1e-4
    else:
        d = np.abs(got.view(np.uint16).astype(np.int32) - ref.astype(np.int32))
        print("p16 max LSB", d.max(), "frac > 0:", (d > 0).mean())
        assert d.max() <= 1


def test_host_pipeline_matches_device(cuda):
    """chdg_decode_host (pinned H2D + decode + D2H in batches of 16, 64 and
    16 frames with the 3D halo, on two device slots) gives the same frames as
    the device-resident decode; a second call issued before the first has
    finished reuses the slots only after the first call's work on them."""
    import ctypes as C
    torch = cuda
    from libchromadec_gb300 import device as D
    cap = capture(200, seed=9)
    n = cap.fields.shape[0]
    nfr = n // 2
    eng = _engine(fmt=0)
    dfields = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    dout = torch.empty((nfr, 3, 576, 948), dtype=torch.int16, device="cuda")
    eng.decode(dfields, 0, nfr, dout)
    ref = dout.cpu()
    hf = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).pin_memory()
    hout = [torch.zeros((nfr, 3, 576, 948), dtype=torch.int16).pin_memory() for _ in range(2)]
    s = torch.cuda.current_stream()
    ranges = [(0, nfr), (3, nfr - 1)]   # back to back, without waiting in between
    for (fb, fe), ho in zip(ranges, hout):
        rc = D.lib().chdg_decode_host(eng._h, C.c_void_p(hf.data_ptr()), hf[0].numel(), n, fb, fe,
                                      C.c_void_p(ho.data_ptr()), C.c_void_p(s.cuda_stream))
        assert rc == 0, D.last_error()
    torch.cuda.synchronize()
    assert torch.equal(hout[0], ref)
    fb, fe = ranges[1]
    assert torch.equal(hout[1][:fe - fb], ref[fb:fe])
