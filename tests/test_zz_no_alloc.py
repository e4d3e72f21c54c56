"""The allocation-free FFT-CN entry point against the workspace version.

``mjx_fft_cn2d_noalloc`` serves hosts that cannot allocate device memory
themselves (for example a driver loop embedded in another runtime whose
allocator owns all device memory, or code that must not call into an
allocator at all): it takes only the input and output buffers and uses a
fixed scratch array that lives inside the library.  These tests call it
through the C ABI, twice in a row with different inputs, and check each
result against ``mjx_fft_cn2d`` with a caller-provided workspace.  The file
sorts last so that a run stopping at the first failure has already run
every other test.
"""

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _plan(ny, nx, dtype, dev):
    from moljax_gb300.core.fft_solvers import get_plan
    return get_plan(ny, nx, 1.0 / ny, 1.0 / nx, "spectral", dtype, dev)


@pytest.mark.parametrize("n,dtype", [(128, torch.float64), (1024, torch.float32)])
def test_noalloc_matches_workspace_version(cuda, native_lib, n, dtype):
    from moljax_gb300 import _native as N
    lib = native_lib
    plan = _plan(n, n, dtype, cuda)
    code = N.dtype_code(dtype)
    ws_bytes = lib.mjx_spec2d_ws_bytes(n, n, 1, code)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    rng = np.random.default_rng(n)
    stream = N.stream_ptr(cuda)
    tol = 1e-13 if dtype == torch.float64 else 1e-6
    for call in range(2):  # two calls in a row share the fixed scratch
        u = torch.tensor(rng.standard_normal((n, n)), dtype=dtype, device=cuda)
        ref = torch.empty_like(u)
        out = torch.full_like(u, float("nan"))
        N.check("mjx_fft_cn2d", lib.mjx_fft_cn2d(
            N.ptr(plan.buf), C.byref(plan.cgrid), code, 0.1, 0.01, 5, N.ptr(u), N.ptr(ref),
            N.ptr(ws), ws.numel(), stream))
        st = lib.mjx_fft_cn2d_noalloc(N.ptr(plan.buf), C.byref(plan.cgrid), code, 0.1, 0.01, 5,
                                      N.ptr(u), N.ptr(out), stream)
        assert st == 0, N.STATUS_NAMES.get(st, st)
        torch.cuda.synchronize(cuda)
        err = float(torch.linalg.norm((out - ref).double()) / torch.linalg.norm(ref.double()))
        assert err < tol, (call, err)


def test_noalloc_rejects_grids_beyond_the_scratch(cuda, native_lib):
    from moljax_gb300 import _native as N
    g = N.Grid2DC(2048, 2048, 1.0 / 2048, 1.0 / 2048)
    # the size check comes before any device access; pointers are never touched
    st = native_lib.mjx_fft_cn2d_noalloc(C.c_void_p(1), C.byref(g), N.F32, 0.1, 0.01, 1,
                                         C.c_void_p(1), C.c_void_p(1), None)
    assert st == 10  # MJX_WORKSPACE
