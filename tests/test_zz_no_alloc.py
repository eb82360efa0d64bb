"""The allocation-free projection entry point (gtn_multidot_noalloc) against numpy's
V.conj() @ w and against the regular gtn_dot entry point, through the C ABI.  It serves callers that cannot let the library
allocate device memory (their own pool owns the GPU's memory, or cudaMalloc's device-wide
synchronisation is unacceptable), so it keeps its partial sums in a fixed library array.
This file is collected last so that a failure here comes after every other test ran."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_multidot_noalloc_matches_dot(ctx):
    import torch
    from grafttn import _lib
    lib = _lib.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(123)
    for call, (J, n) in enumerate([(7, 100003), (64, 4099)]):  # two calls in a row
        V = (rng.standard_normal((J, n)) + 1j * rng.standard_normal((J, n))) / np.sqrt(2)
        w = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) / np.sqrt(2)
        dV, dw = ctx.upload(V), ctx.upload(w)
        out = ctx.empty((J,))
        st = lib.gtn_multidot_noalloc(stream, n, J, C.c_void_p(dV.data_ptr()), n, C.c_void_p(dw.data_ptr()),
                                      C.c_void_p(out.data_ptr()))
        assert st == _lib.GTN_OK
        torch.cuda.synchronize()
        got = ctx.download(out)
        tol = 1e-12 * np.linalg.norm(V, axis=1) * np.linalg.norm(w)
        exact = V.conj() @ w                                      # numpy, complex128
        assert np.all(np.abs(got - exact) <= tol), (call, np.max(np.abs(got - exact)))
        ref = np.array([ctx.dot(dV[j], dw) for j in range(J)])   # the existing entry point
        assert np.all(np.abs(got - ref) <= tol), (call, np.max(np.abs(got - ref)))


def test_multidot_noalloc_rejects_sizes_beyond_limit(ctx):
    import torch
    from grafttn import _lib
    lib = _lib.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    x = ctx.empty((65, 8))
    out = ctx.empty((65,))
    assert lib.gtn_multidot_noalloc(stream, 8, 65, C.c_void_p(x.data_ptr()), 8, C.c_void_p(x.data_ptr()),
                                    C.c_void_p(out.data_ptr())) == _lib.GTN_ERR_INVALID
    assert lib.gtn_multidot_noalloc(stream, 8, 0, C.c_void_p(x.data_ptr()), 8, C.c_void_p(x.data_ptr()),
                                    C.c_void_p(out.data_ptr())) == _lib.GTN_ERR_INVALID
