"""Batches of captures (chdg_batch_*): many captures of uneven length, mixed
Transform-PAL 2D/3D, one threshold each, decoded by one launch per mode and
replayed from a CUDA graph. Every frame must equal the single-capture decode
of its own capture bit for bit (the batch's black gaps are the reference's
window padding), through the eager run, the graph capture, the replays and
after autotuning; sampled frames also against the CPU oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from tests._capture import capture

pytestmark = pytest.mark.gpu


def test_batch_equals_per_capture_decode(cuda):
    torch = cuda
    from libchromadec_gb300 import device as D
    rng = np.random.default_rng(12)
    lengths = [2, 30, 6, 16, 3, 24, 8, 2, 12, 5]          # fields (odd ones leave an unpaired last field)
    kinds = [8, 8, 7, 8, 7, 8, 7, 8, 8, 7]
    thr = rng.uniform(0.3, 0.6, len(lengths))
    src = capture(40, 61, dropouts=0.0)
    caps, refs = [], []
    for i, (n, k) in enumerate(zip(lengths, kinds)):
        start = int(rng.integers(0, 40 - n + 1))
        f = torch.from_numpy(np.ascontiguousarray(src.fields[start:start + n]).reshape(n, -1).view(np.int16)).cuda()
        out = torch.zeros((n // 2, 3, 576, 948), dtype=torch.int16, device="cuda")
        caps.append((f, k, float(thr[i]), out))
        eng = D.Engine(D.default_geometry(), D.default_config(kind=k, fmt=D.FMT_P16, threshold=float(thr[i])))
        ref = torch.empty_like(out)
        eng.decode(f, 0, n // 2, ref)
        refs.append(ref)
    s = torch.cuda.Stream()
    b = D.Batch(D.default_geometry(), D.default_config(kind=8, fmt=D.FMT_P16))
    arr = D.Batch.captures(caps)
    for rep in range(4):                                   # eager, capture, replay, replay
        for _, _, _, out in caps:
            out.zero_()
        torch.cuda.synchronize()
        b.decode(arr, s)
        s.synchronize()
        for (f, k, t, out), ref in zip(caps, refs):
            assert torch.equal(out, ref), (rep, k, f.shape[0])
    tuning = b.autotune(arr, s)
    assert tuning.chunk_frames in (16, 24, 32, 48, 64) and tuning.ms > 0
    for rep in range(3):
        for _, _, _, out in caps:
            out.zero_()
        b.decode(arr, s)
        s.synchronize()
        for (f, k, t, out), ref in zip(caps, refs):
            assert torch.equal(out, ref), ("tuned", rep)
    # oracle parity on a sampled 3D and 2D capture
    for idx in (1, 5, 2):
        f, k, t, out = caps[idx]
        fields = f.cpu().numpy().view(np.uint16).reshape(f.shape[0], 313, 1135)
        n = f.shape[0] // 2
        ref, _ = O.decode_frames(O.params(3 if k == 8 else 2, O.FMT_P16, threshold=t), fields, 0, n, threads=8)
        d = np.abs(out.cpu().numpy().view(np.uint16).astype(np.int32) - ref.astype(np.int32))
        assert d.max() <= 1
    b.close()
