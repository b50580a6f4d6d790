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


def test_batch_conceals_and_masks_dropouts(cuda):
    """Captures with 2 % dropout lines, concealed inside the batch (single-frame
    plans, every mode) and masked: each frame equals the engine's decode of
    the capture concealed by the oracle's DropoutCorrector (itself byte-exact
    with the reference's), bit for bit; masks equal the oracle's spans
    rastered; the caller's fields are left as they were; eager, captured and
    replayed decodes agree."""
    torch = cuda
    from libchromadec_gb300 import device as D, synth
    specs = [(12, 8, D.CONCEAL), (7, 7, D.CONCEAL | D.CONCEAL_OVERCORRECT), (20, 8, D.CONCEAL | D.CONCEAL_INTRA),
             (6, 7, 0), (9, 8, D.CONCEAL | D.CONCEAL_OVERCORRECT | D.CONCEAL_INTRA)]
    items, refs, masks_ref, originals = [], [], [], []
    for i, (n, kind, flags) in enumerate(specs):
        cap = synth.make_capture(n, synth.SynthConfig(seed=90 + i, pan_x=1.0 + 0.5 * i, pan_y=0.5,
                                                      dropout_line_fraction=0.02))
        drops = O.flatten_dropouts(cap.dropouts)
        assert drops
        p = O.params(3 if kind == 8 else 2, O.FMT_P16)
        conc = cap.fields.copy()
        if flags & D.CONCEAL:
            for k in range(n // 2):
                conc[2 * k:2 * k + 2], _ = O.dropout_correct_frame(p, cap.fields, k, drops,
                                                                   overcorrect=bool(flags & D.CONCEAL_OVERCORRECT),
                                                                   intra=bool(flags & D.CONCEAL_INTRA))
        f = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
        fc = torch.from_numpy(conc.reshape(n, -1).view(np.int16)).cuda()
        eng = D.Engine(D.default_geometry(), D.default_config(kind=kind, fmt=D.FMT_P16))
        ref = torch.empty((n // 2, 3, 576, 948), dtype=torch.int16, device="cuda")
        # an unpaired last field belongs to no frame: the batch, like the
        # reference's window, reads it as black, so the reference decode gets
        # the whole frames only
        eng.decode(fc[:2 * (n // 2)], 0, n // 2, ref)
        refs.append(ref)
        mref = np.zeros((n // 2, 576, 948), dtype=np.uint16)
        for k in range(n // 2):
            for y, x0, x1, _ in O.dropout_spans(p, drops, k, 0):
                mref[k, y, x0:x1] = 0xFFFF
        masks_ref.append(mref)
        out = torch.zeros_like(ref)
        mask = torch.full((n // 2, 576, 948), 7, dtype=torch.int16, device="cuda")
        items.append((f, kind, 0.4, out, drops, flags, mask))
        originals.append(f.clone())
    s = torch.cuda.Stream()
    b = D.Batch(D.default_geometry(), D.default_config(kind=8, fmt=D.FMT_P16))
    arr = D.Batch.captures(items)
    for rep in range(3):                                   # eager, capture, replay
        for it in items:
            it[3].zero_()
            it[6].fill_(7)
        torch.cuda.synchronize()
        b.decode(arr, s)
        s.synchronize()
        for i, (it, ref, mref, orig) in enumerate(zip(items, refs, masks_ref, originals)):
            assert torch.equal(it[3], ref), (rep, i)
            assert np.array_equal(it[6].cpu().numpy().view(np.uint16), mref), (rep, i)
            assert torch.equal(it[0], orig), (rep, i)
    b.close()
