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
