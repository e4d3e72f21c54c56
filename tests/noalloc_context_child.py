"""Child process of ``test_zz_no_alloc.py``: the allocation-free FFT-CN entry
point in two CUDA contexts of one process.

A host that embeds this library inside another runtime often drives the GPU
through the CUDA driver API with a context of its own rather than the
device's primary context.  A ``__device__`` array has a different address in
every context that loads the library, so the entry point must look the
scratch address up for the context that is current when it is called.  This
script runs ``mjx_fft_cn2d_noalloc`` against ``mjx_fft_cn2d`` first in the
primary context, then in a context created with ``cuCtxCreate``, then in the
primary context again.  It uses only ctypes (no torch), and the test process
(not the entry point) allocates the buffers with ``cuMemAlloc``.

Usage: python noalloc_context_child.py <path of libmoljax_gb300.so>
Prints ``OK <max relative error>`` and exits 0 when every case matches.
"""

import ctypes as C
import sys

import numpy as np


class Grid2D(C.Structure):
    _fields_ = [("ny", C.c_int), ("nx", C.c_int), ("dy", C.c_double), ("dx", C.c_double)]


def main(lib_path):
    lib = C.CDLL(lib_path)
    cu = C.CDLL("libcuda.so.1")
    P, D, I, S = C.c_void_p, C.c_double, C.c_int, C.c_size_t
    lib.mjx_spec2d_plan_bytes.restype = S
    lib.mjx_spec2d_plan_bytes.argtypes = [I, I, I]
    lib.mjx_spec2d_ws_bytes.restype = S
    lib.mjx_spec2d_ws_bytes.argtypes = [I, I, I, I]
    lib.mjx_spec2d_plan_init.argtypes = [P, C.POINTER(Grid2D), I, I, P]
    lib.mjx_fft_cn2d.argtypes = [P, C.POINTER(Grid2D), I, D, D, I, P, P, P, S, P]
    lib.mjx_fft_cn2d_noalloc.argtypes = [P, C.POINTER(Grid2D), I, D, D, I, P, P, P]
    cu.cuMemAlloc_v2.argtypes = [C.POINTER(C.c_uint64), S]
    cu.cuMemFree_v2.argtypes = [C.c_uint64]
    cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, P, S]
    cu.cuMemcpyDtoH_v2.argtypes = [P, C.c_uint64, S]

    def ck(r, what):
        if r != 0:
            raise RuntimeError(f"{what} returned {r}")

    def alloc(nbytes):
        d = C.c_uint64()
        ck(cu.cuMemAlloc_v2(C.byref(d), nbytes), "cuMemAlloc")
        return d.value

    def case(n, dtype_code, seed):
        npdt = np.float32 if dtype_code == 0 else np.float64
        g = Grid2D(n, n, 1.0 / n, 1.0 / n)
        plan = alloc(lib.mjx_spec2d_plan_bytes(n, n, dtype_code))
        ws_bytes = lib.mjx_spec2d_ws_bytes(n, n, 1, dtype_code)
        ws = alloc(ws_bytes)
        nb = n * n * np.dtype(npdt).itemsize
        u, ref, out = alloc(nb), alloc(nb), alloc(nb)
        try:
            ck(lib.mjx_spec2d_plan_init(P(plan), C.byref(g), 1, dtype_code, None), "plan_init")
            host = np.random.default_rng(seed).standard_normal((n, n)).astype(npdt)
            ck(cu.cuMemcpyHtoD_v2(u, host.ctypes.data, nb), "HtoD")
            ck(lib.mjx_fft_cn2d(P(plan), C.byref(g), dtype_code, 0.1, 0.01, 5, P(u), P(ref), P(ws),
                                ws_bytes, None), "mjx_fft_cn2d")
            ck(lib.mjx_fft_cn2d_noalloc(P(plan), C.byref(g), dtype_code, 0.1, 0.01, 5, P(u), P(out),
                                        None), "mjx_fft_cn2d_noalloc")
            ck(cu.cuCtxSynchronize(), "cuCtxSynchronize")
            a, b = np.empty_like(host), np.empty_like(host)
            ck(cu.cuMemcpyDtoH_v2(a.ctypes.data, ref, nb), "DtoH")
            ck(cu.cuMemcpyDtoH_v2(b.ctypes.data, out, nb), "DtoH")
            err = float(np.linalg.norm((b - a).astype(np.float64)) / np.linalg.norm(a.astype(np.float64)))
            tol = 1e-6 if dtype_code == 0 else 1e-13
            if not err < tol:
                raise AssertionError(f"n={n} dtype={dtype_code}: rel err {err}")
            return err
        finally:
            for d in (plan, ws, u, ref, out):
                cu.cuMemFree_v2(d)

    ck(cu.cuInit(0), "cuInit")
    dev = I()
    ck(cu.cuDeviceGet(C.byref(dev), 0), "cuDeviceGet")
    primary = P()
    ck(cu.cuDevicePrimaryCtxRetain(C.byref(primary), dev), "cuDevicePrimaryCtxRetain")
    ck(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
    errs = [case(128, 1, 1), case(256, 0, 2)]
    second = P()
    ck(cu.cuCtxCreate_v2(C.byref(second), 0, dev), "cuCtxCreate")  # now current
    errs += [case(128, 1, 3), case(256, 0, 4)]
    ck(cu.cuCtxDestroy_v2(second), "cuCtxDestroy")
    ck(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
    errs += [case(128, 1, 5)]
    ck(cu.cuDevicePrimaryCtxRelease_v2(dev), "cuDevicePrimaryCtxRelease")
    print("OK", max(errs))


if __name__ == "__main__":
    main(sys.argv[1])
