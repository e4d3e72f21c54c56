"""The allocation-free FFT-CN entry point against the workspace version.

``mjx_fft_cn2d_noalloc`` serves hosts that cannot allocate device memory
themselves (for example a driver loop embedded in another runtime whose
allocator owns all device memory, or code that must not call into an
allocator at all): it takes only the input and output buffers and uses a
fixed scratch array that lives inside the library.  These tests call it
through the C ABI, twice in a row with different inputs, and check each
result against ``mjx_fft_cn2d`` with a caller-provided workspace; they also
pin the size limit on both sides, an in-place call, and calls from a second
CUDA context of the same process.  The file sorts last so that a run
stopping at the first failure has already run every other test.
"""

import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SCRATCH = 8 << 20  # MJX_NOALLOC_SCRATCH_BYTES


def _plan(ny, nx, dtype, dev):
    from moljax_gb300.core.fft_solvers import get_plan
    return get_plan(ny, nx, 1.0 / ny, 1.0 / nx, "spectral", dtype, dev)


def _compare(lib, cuda, ny, nx, dtype, seed, in_place=False):
    from moljax_gb300 import _native as N
    plan = _plan(ny, nx, dtype, cuda)
    code = N.dtype_code(dtype)
    ws_bytes = lib.mjx_spec2d_ws_bytes(ny, nx, 1, code)
    assert ws_bytes <= SCRATCH
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda)
    rng = np.random.default_rng(seed)
    stream = N.stream_ptr(cuda)
    tol = 1e-13 if dtype == torch.float64 else 1e-6
    for call in range(2):  # two calls in a row share the fixed scratch
        u = torch.tensor(rng.standard_normal((ny, nx)), dtype=dtype, device=cuda)
        ref = torch.empty_like(u)
        N.check("mjx_fft_cn2d", lib.mjx_fft_cn2d(
            N.ptr(plan.buf), C.byref(plan.cgrid), code, 0.1, 0.01, 5, N.ptr(u), N.ptr(ref),
            N.ptr(ws), ws.numel(), stream))
        if in_place:
            out = u.clone()
            src = out
        else:
            out = torch.full_like(u, float("nan"))
            src = u
        st = lib.mjx_fft_cn2d_noalloc(N.ptr(plan.buf), C.byref(plan.cgrid), code, 0.1, 0.01, 5,
                                      N.ptr(src), N.ptr(out), stream)
        assert st == 0, N.STATUS_NAMES.get(st, st)
        torch.cuda.synchronize(cuda)
        err = float(torch.linalg.norm((out - ref).double()) / torch.linalg.norm(ref.double()))
        assert err < tol, (call, err)


@pytest.mark.parametrize("n,dtype", [(128, torch.float64), (1024, torch.float32),
                                     (512, torch.float64)])
def test_noalloc_matches_workspace_version(cuda, native_lib, n, dtype):
    # 1024^2 FP32 and 512^2 FP64 are the largest square grids the 8 MiB scratch holds
    _compare(native_lib, cuda, n, n, dtype, n)


@pytest.mark.parametrize("ny,nx", [(512, 2048), (2048, 512)])
def test_noalloc_non_square(cuda, native_lib, ny, nx):
    _compare(native_lib, cuda, ny, nx, torch.float32, ny + nx)


def test_noalloc_in_place(cuda, native_lib):
    _compare(native_lib, cuda, 256, 256, torch.float64, 7, in_place=True)


@pytest.mark.parametrize("n,dtype", [(2048, 0), (1024, 1)])
def test_noalloc_rejects_grids_beyond_the_scratch(cuda, native_lib, n, dtype):
    from moljax_gb300 import _native as N
    assert native_lib.mjx_spec2d_ws_bytes(n, n, 1, dtype) > SCRATCH
    g = N.Grid2DC(n, n, 1.0 / n, 1.0 / n)
    # the size check comes before any device access; pointers are never touched
    st = native_lib.mjx_fft_cn2d_noalloc(C.c_void_p(1), C.byref(g), dtype, 0.1, 0.01, 1,
                                         C.c_void_p(1), C.c_void_p(1), None)
    assert st == 10  # MJX_WORKSPACE


def test_noalloc_in_a_second_context(cuda, native_lib):
    """A driver-API context of its own (as an embedding runtime may hold) gets
    the scratch address of that context, not the primary context's."""
    from moljax_gb300.build_native import LIB
    child = os.path.join(os.path.dirname(os.path.abspath(__file__)), "noalloc_context_child.py")
    r = subprocess.run([sys.executable, child, LIB], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.startswith("OK"), r.stdout + r.stderr
