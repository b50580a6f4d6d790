"""The allocation-free decode entry point (chdg_decode_device_static).

Some callers cannot allocate device memory while decoding (their device
memory is owned by their own allocator or budget, or cudaMalloc's implicit
synchronisation would stall a latency-critical loop). For them the library
exports a decode whose chroma scratch is a static device array. This test
calls it through the C ABI twice in a row -- the second call reuses the
scratch the first one left behind -- and checks both results against the
regular entry point (chdg_decode_device), which allocates its scratch.
It is kept in a file collected last so a failure here cannot hide other
results; it passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from tests._capture import capture

pytestmark = pytest.mark.gpu


def test_static_scratch_decode_matches_allocating_decode(cuda):
    torch = cuda
    from libchromadec_gb300 import device as D

    lib = D.lib()
    lib.chdg_decode_device_static.argtypes = [C.POINTER(D.Geometry), C.POINTER(D.Config), C.c_void_p, C.c_int64,
                                              C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    cap = capture(24, seed=13)
    n = cap.fields.shape[0]
    fields = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    for fmt, dt in ((D.FMT_P16, torch.int16), (D.FMT_PS, torch.float32)):
        g = D.default_geometry()
        c = D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=fmt)
        eng = D.Engine(g, c)
        stream = torch.cuda.current_stream()
        # two consecutive calls, different frame ranges, shared scratch
        for fb, fe in ((0, 8), (3, 9)):
            ref = torch.empty((fe - fb, 3, 576, 948), dtype=dt, device="cuda")
            eng.decode(fields, fb, fe, ref, stream)
            got = torch.full((fe - fb, 3, 576, 948), 7, dtype=dt, device="cuda")
            rc = lib.chdg_decode_device_static(C.byref(g), C.byref(c), C.c_void_p(fields.data_ptr()),
                                               fields[0].numel(), n, fb, fe, C.c_void_p(got.data_ptr()),
                                               C.c_void_p(stream.cuda_stream))
            assert rc == 0, D.last_error()
            torch.cuda.synchronize()
            if fmt == D.FMT_PS:
                assert float((got - ref).abs().max()) <= 1e-6
            else:
                assert torch.equal(got, ref)
        eng.close()


def _static_fn(D):
    lib = D.lib()
    fn = lib.chdg_decode_device_static
    fn.argtypes = [C.POINTER(D.Geometry), C.POINTER(D.Config), C.c_void_p, C.c_int64, C.c_int32, C.c_int32,
                   C.c_int32, C.c_void_p, C.c_void_p]
    return fn


def test_static_per_bin_tables_back_to_back_on_a_non_blocking_stream(cuda):
    """Two calls in a row with different per-bin threshold tables, queued on
    one non-blocking stream without a host wait between them: the second
    call's table upload must not overtake the first call's kernels."""
    torch = cuda
    from libchromadec_gb300 import device as D

    fn = _static_fn(D)
    cap = capture(20, seed=17)
    n = cap.fields.shape[0]
    fields = torch.from_numpy(cap.fields.reshape(n, -1).view(np.int16)).cuda()
    rng = np.random.default_rng(3)
    tables = [rng.uniform(0.25, 0.55, 768), rng.uniform(0.35, 0.65, 768)]
    stream = torch.cuda.Stream()   # created non-blocking with respect to the legacy stream
    assert stream.cuda_stream != 0
    g = D.default_geometry()
    cfgs = [D.default_config(kind=D.KIND_TRANSFORM_3D, fmt=D.FMT_P16, thresholds=list(t)) for t in tables]
    outs, refs = [], []
    for c in cfgs:
        eng = D.Engine(g, c)
        ref = torch.empty((6, 3, 576, 948), dtype=torch.int16, device="cuda")
        eng.decode(fields, 1, 7, ref)
        torch.cuda.synchronize()
        refs.append(ref)
        eng.close()
    assert not torch.equal(refs[0], refs[1])          # the tables make a difference
    with torch.cuda.stream(stream):
        outs = [torch.full((6, 3, 576, 948), 3, dtype=torch.int16, device="cuda") for _ in cfgs]
        for i, c in enumerate(cfgs):
            rc = fn(C.byref(g), C.byref(c), C.c_void_p(fields.data_ptr()), fields[0].numel(), n, 1, 7,
                    C.c_void_p(outs[i].data_ptr()), C.c_void_p(stream.cuda_stream))
            assert rc == 0, D.last_error()
    stream.synchronize()
    for i in range(2):
        assert torch.equal(outs[i], refs[i]), i


def test_static_scratch_decode_rejects_oversize(cuda):
    torch = cuda
    from libchromadec_gb300 import device as D

    lib = D.lib()
    lib.chdg_decode_device_static.argtypes = [C.POINTER(D.Geometry), C.POINTER(D.Config), C.c_void_p, C.c_int64,
                                              C.c_int32, C.c_int32, C.c_int32, C.c_void_p, C.c_void_p]
    g = D.default_geometry()
    c = D.default_config(kind=D.KIND_TRANSFORM_3D)
    dummy = torch.zeros(16, dtype=torch.int16, device="cuda")
    rc = lib.chdg_decode_device_static(C.byref(g), C.byref(c), C.c_void_p(dummy.data_ptr()), 1135 * 313, 40, 0, 9,
                                       C.c_void_p(dummy.data_ptr()), None)
    assert rc == -1
    assert "at most 8 frames" in D.last_error()
    # a negative start or a reversed range
    for fb, fe in ((-1, 3), (5, 4), (-2147483647, 2147483647)):
        rc = lib.chdg_decode_device_static(C.byref(g), C.byref(c), C.c_void_p(dummy.data_ptr()), 1135 * 313, 40,
                                           fb, fe, C.c_void_p(dummy.data_ptr()), None)
        assert rc == -1, (fb, fe)
        assert "frame" in D.last_error()
    # an active picture larger than the static planes hold
    big = D.default_geometry()
    big.first_active_frame_line = 20
    big.last_active_frame_line = 621
    rc = lib.chdg_decode_device_static(C.byref(big), C.byref(c), C.c_void_p(dummy.data_ptr()), 1135 * 313, 40, 0, 8,
                                       C.c_void_p(dummy.data_ptr()), None)
    assert rc == -1
    assert "too large" in D.last_error()
