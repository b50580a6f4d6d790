"""CPU restatement of the tensor-core mask network's data layout and
schedule (mn_tc_forward_kernel, libchromadec_gb300/csrc/masknet.cu), checked
against the FP64 forward pass (tests/masknet_ref.py).

The GPU tests (test_gpu_masknet.py) check the CUDA kernel's results; this
test checks the design they rest on, in numpy:

  * the weight images as mn_build_images_kernel lays them out (layer 1
    [dy][240 rows (q, dz, co)][K 16]; layers 2 and 3 [chunk][dy][band rows]
    [K 16]), each tap's image in the no-swizzle K-major canonical layout;
  * every MMA's operands read through the shared-memory descriptor rule
    (8-row core matrices of 16 bytes a row, K-adjacent ones 128 bytes apart,
    row groups SBO apart), at the start addresses the kernel computes;
  * the banded chunks' output columns, accumulation into columns the
    epilogue cleared, and the lane-shuffle sum of the kz partials;
  * the schedule's hazards: every 16-byte chunk of the operand regions is
    tagged with the layer (and tile) that wrote it and each MMA checks the
    tags it reads. The MMAs run at the two ends of what the barriers allow:
    eagerly (a block-0 chunk as soon as block 1's step q releases it; block
    1's chunks only after block 0's whole epilogue, which overlaps them on the
    GPU), and lazily (every chunk of an M block just before the block's
    epilogue, whose barrier is committed after the block's last chunk).

Two planted mistakes must be caught: block 0's epilogue writing its stashed
rows in place (the tag check), and a block's barrier committed before its
last chunk (the result).
"""
import numpy as np
import pytest

from tests import masknet_ref as R

NCOL = 240
GROUPS = 34
A_BYTES = GROUPS * 8 * 160
IN_BYTES = GROUPS * 8 * 32
OFF_B1 = 27 * 2 * 16
OFF_B2 = OFF_B1 + 16 + 27 * 256
OFF_B3 = OFF_B2 + 16 + 27 * 256
OFF_WH = OFF_B3 + 16
OFF_BH = OFF_WH + 16
OFF_W = {1: 0, 2: OFF_B1 + 16, 3: OFF_B2 + 16}


def band_lo(ks):
    return ks - 1 if ks > 0 else 0


def band_q(ks):
    return (ks + 1 if ks < 4 else 4) - band_lo(ks) + 1


def band_off(ks):
    return sum(3 * 48 * band_q(k) * 32 for k in range(ks))


IMG_L1 = 0
IMG_L2 = 3 * NCOL * 32
IMG_L3 = IMG_L2 + band_off(5)
IMG_BYTES = IMG_L3 + band_off(5)


def elem_off(r, k):
    """Byte offset of bf16 element k of row r, rows of 32 bytes (K = 16)."""
    kb = 2 * k
    return (r >> 3) * 256 + (kb >> 4) * 128 + (r & 7) * 16 + (kb & 15)


def bf16_bits(x):
    a = np.ascontiguousarray(x, dtype=np.float32).reshape(-1)
    u = a.view(np.uint32).astype(np.uint64)
    return ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)


def from_bits(b):
    return (np.asarray(b, dtype=np.uint32) << 16).view(np.float32).astype(np.float64)


def build_images(used):
    """mn_build_images_kernel's layout, element by element."""
    img = np.zeros(IMG_BYTES // 2, dtype=np.uint16)
    for dy in range(3):
        for n in range(NCOL):
            q, dz, co = n // 48, (n % 48) >> 4, n & 15
            for k in range(10):
                dq, ci = k // 2 - q, k % 2
                if -1 <= dq <= 1:
                    v = used[OFF_W[1] + (((dz * 3 + dy) * 3 + dq + 1) * 2 + ci) * 16 + co]
                    img[(IMG_L1 + dy * NCOL * 32 + elem_off(n, k)) // 2] = bf16_bits([v])[0]
    for layer, base in ((2, IMG_L2), (3, IMG_L3)):
        for ks in range(5):
            nb = 48 * band_q(ks)
            for dy in range(3):
                for n in range(nb):
                    nn = 48 * band_lo(ks) + n
                    q, dz, co = nn // 48, (nn % 48) >> 4, nn & 15
                    dq = ks - q
                    assert -1 <= dq <= 1
                    for k in range(16):
                        v = used[OFF_W[layer] + (((dz * 3 + dy) * 3 + dq + 1) * 16 + k) * 16 + co]
                        off = base + band_off(ks) + dy * nb * 32 + elem_off(n, k)
                        img[off // 2] = bf16_bits([v])[0]
    return img


class Region:
    """Shared-memory bytes as bf16 halves, with a writer tag per 16-byte chunk."""

    def __init__(self, nbytes):
        self.v = np.zeros(nbytes // 2, dtype=np.uint16)
        self.tag = np.full(nbytes // 16, -1, dtype=np.int64)

    def put(self, off, v8, tag):
        assert off % 16 == 0 and 0 <= off and off + 16 <= self.v.size * 2
        self.v[off // 2:off // 2 + 8] = v8
        self.tag[off // 16] = tag

    def operand(self, start, sbo, rows, want_tag=None):
        m = np.arange(rows)[:, None]
        k = np.arange(16)[None, :]
        addr = start + (m >> 3) * sbo + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2
        assert addr.min() >= 0 and addr.max() + 2 <= self.v.size * 2
        if want_tag is not None:
            tags = self.tag[addr // 16]
            assert (tags == want_tag).all(), f"operand written by {np.unique(tags)}, expected {want_tag}"
        return from_bits(self.v[addr // 2])


def put_row(reg, row_bytes, ky, kz, c, v8, tag):
    grp = 8 * row_bytes
    base = c * 128 + kz * 16
    reg.put(base + (ky + 1) * grp, v8, tag)
    if ky == 31:
        reg.put(base, v8, tag)
    if ky == 0:
        reg.put(base + (GROUPS - 1) * grp, v8, tag)


def final_chunk(q):
    """The chunk after which output block q may be read: an M block's one
    barrier is committed after its last chunk (4), although chunk ks writes
    only the output blocks ks - 1 .. ks + 1."""
    return 4


def run(used, img, feats, plant_hazard=False, lazy=False, last_chunk=final_chunk):
    """The kernel's schedule over consecutive tiles of one CTA; fractions per tile."""
    A, IN = Region(A_BYTES), Region(IN_BYTES)
    W1 = Region(3 * NCOL * 32)
    W1.v[:] = img[IMG_L1 // 2:(IMG_L1 + 3 * NCOL * 32) // 2]
    stash = {}
    tm = [np.full((128, NCOL), np.nan), np.full((128, NCOL), np.nan)]   # each M block's columns

    def piece(layer, ks):
        off = (IMG_L2 if layer == 2 else IMG_L3) + band_off(ks)
        nbytes = 3 * 48 * band_q(ks) * 32
        reg = Region(nbytes)
        reg.v[:] = img[off // 2:(off + nbytes) // 2]
        return reg

    def write_input(tj):
        f = feats[tj]
        for r in range(256):
            ky, kz = r >> 3, r & 7
            v = np.zeros(16, dtype=np.uint16)
            for q in range(5):
                v[2 * q] = f[(q * 8 + kz) * 32 + ky]
                v[2 * q + 1] = f[((4 - q) * 8 + ((10 - kz) & 7)) * 32 + ((40 - ky) & 31)]
            put_row(IN, 32, ky, kz, 0, v[:8], 100 + tj)
            put_row(IN, 32, ky, kz, 1, v[8:], 100 + tj)

    def mma_layer1(b, tj):
        for dy in range(3):
            d = IN.operand((b * 16 + dy) * 256, 256, 128, 100 + tj) @ W1.operand(dy * NCOL * 32, 256, NCOL).T
            tm[b][:, :] = d if dy == 0 else tm[b] + d

    def mma_chunk(layer, b, ks, tj):
        nb, lo = 48 * band_q(ks), 48 * band_lo(ks)
        P = piece(layer, ks)
        for dy in range(3):
            a = A.operand((b * 16 + dy) * 1280 + ks * 256, 1280, 128, 10 * tj + layer - 1)
            blk = tm[b][:, lo:lo + nb]
            assert not np.isnan(blk).any(), "accumulating into columns nobody cleared"
            tm[b][:, lo:lo + nb] = blk + a @ P.operand(dy * nb * 32, 256, nb).T

    pending = {0: [], 1: []}   # issued chunks not yet executed, in issue order

    def issue(layer, b, ks, tj):
        if lazy:
            pending[b].append((layer, ks, tj))
        else:
            mma_chunk(layer, b, ks, tj)

    def need(b, q, everything=False):
        """Output block q's wait: the chunks up to last_chunk(q) have completed
        (everything: the block's epilogue is over and the rest complete too)."""
        while pending[b] and (everything or pending[b][0][1] <= last_chunk(q)):
            layer, ks, tj = pending[b].pop(0)
            mma_chunk(layer, b, ks, tj)

    def combine(b, q):
        D = tm[b]
        y = np.zeros((128, 16))
        for lr in range(128):
            kz = lr & 7
            lm, lp = (lr & ~7) | ((kz - 1) & 7), (lr & ~7) | ((kz + 1) & 7)
            y[lr] = D[lm, q * 48:q * 48 + 16] + D[lr, q * 48 + 16:q * 48 + 32] + D[lp, q * 48 + 32:q * 48 + 48]
        return y

    def epi_step(layer, b, q, tj):
        need(b, q)
        y = combine(b, q)
        tm[b][:, q * 48:q * 48 + 48] = 0.0   # cleared after reading: the next layer accumulates
        bias = used[(OFF_B1 if layer == 1 else OFF_B2):][:16]
        tag = 10 * tj + layer
        for lr in range(128):
            ky, kz = (b * 128 + lr) >> 3, lr & 7
            o = bf16_bits(np.maximum(y[lr] + bias, 0.0))
            for h in range(2):
                ch, v8 = 2 * q + h, o[8 * h:8 * h + 8]
                if b == 0:
                    if ky == 15 and not plant_hazard:
                        stash[(0, kz, ch)] = v8
                    else:
                        A.put((ky + 1) * 1280 + ch * 128 + kz * 16, v8, tag)
                    if ky == 0:
                        stash[(1, kz, ch)] = v8
                else:
                    put_row(A, 160, ky, kz, ch, v8, tag)
                    if ky == 16:
                        A.put(33 * 1280 + ch * 128 + kz * 16, stash[(1, kz, ch)], tag)
                    if ky == 31 and not plant_hazard:
                        A.put(16 * 1280 + ch * 128 + kz * 16, stash[(0, kz, ch)], tag)

    def head(b, p):
        for q in range(5):
            need(b, q)
            y = combine(b, q)
            for lr in range(128):
                ky, kz = (b * 128 + lr) >> 3, lr & 7
                a = from_bits(bf16_bits(np.maximum(y[lr] + used[OFF_B3:OFF_B3 + 16], 0.0)))
                zh = used[OFF_BH] + (a * used[OFF_WH:OFF_WH + 16]).sum()
                p[(q * 8 + kz) * 32 + ky] = 1.0 / (1.0 + np.exp(-zh))
        need(b, 4, everything=True)

    out = []
    write_input(0)
    for tj in range(len(feats)):
        p = np.zeros(R.NV)
        mma_layer1(0, tj)
        for q in range(5):
            epi_step(1, 0, q, tj)                 # block 0's epilogue before block 1's MMAs
        mma_layer1(1, tj)
        for layer in (2, 3):
            for q in range(5):
                epi_step(layer - 1, 1, q, tj)     # block 1's step q releases chunk q
                issue(layer, 0, q, tj)
            need(1, 4, everything=True)
            if lazy:
                for q in range(5):                # issued right after block 0's
                    issue(layer, 1, q, tj)
            if layer == 2:
                for q in range(5):
                    epi_step(2, 0, q, tj)
                need(0, 4, everything=True)
            else:
                head(0, p)
                if tj + 1 < len(feats):
                    write_input(tj + 1)           # during block 0's head
            if not lazy:
                for q in range(5):
                    issue(layer, 1, q, tj)
        head(1, p)
        out.append(p)
    return out


@pytest.fixture(scope="module")
def problem():
    rng = np.random.default_rng(4)
    used = from_bits(bf16_bits(R.init_params(7)))   # the weights as the network uses them (bf16)
    img = build_images(used)
    X = rng.standard_normal((3, 5, 8, 32)) * 30 + 1j * rng.standard_normal((3, 5, 8, 32)) * 30
    feat = R.features(X)
    return used, img, feat


@pytest.mark.parametrize("lazy", [False, True])
def test_schedule_reproduces_the_fp64_forward(problem, lazy):
    used, img, feat = problem
    got = run(used, img, [bf16_bits(feat[i]) for i in range(3)], lazy=lazy)
    ref, _ = R.forward(used.astype(np.float32), feat)
    for i in range(3):
        assert np.abs(got[i] - ref[i].reshape(-1)).max() < 1e-12


@pytest.mark.parametrize("lazy", [False, True])
def test_planted_hazard_is_caught(problem, lazy):
    used, img, feat = problem
    with pytest.raises(AssertionError, match="operand written by"):
        run(used, img, [bf16_bits(feat[i]) for i in range(2)], plant_hazard=True, lazy=lazy)


def test_block_signalled_early_is_caught(problem):
    """Chunk 4 then completes after the epilogue has read its columns and
    rewritten its operand: the tag check or the results must show it."""
    used, img, feat = problem
    try:
        got = run(used, img, [bf16_bits(feat[i]) for i in range(2)], lazy=True, last_chunk=lambda q: 3)
    except AssertionError as e:
        assert "operand written by" in str(e)
        return
    ref, _ = R.forward(used.astype(np.float32), feat)
    assert np.abs(got[0] - ref[0].reshape(-1)).max() > 1e-3
