"""ctypes binding of ``libmoljax_gb300.so`` (C ABI in ``include/moljax_gb300.h``).

The library is loaded from ``moljax_gb300/_lib`` (built in-tree by
``moljax_gb300.build_native``).  There is no fallback: when the library is
missing or CUDA is unavailable every entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import torch

from moljax_gb300.build_native import LIB

_lock = threading.Lock()
_lib = None

MJX_OK = 0
STATUS_NAMES = {
    0: "MJX_OK", 1: "MJX_BAD_SHAPE", 2: "MJX_BAD_DTYPE", 3: "MJX_NOT_FINITE",
    4: "MJX_MAX_ITERS", 5: "MJX_DT_TOO_SMALL", 6: "MJX_NK_FAILED", 7: "MJX_OOM",
    8: "MJX_CUDA_ERROR", 9: "MJX_BAD_ARG", 10: "MJX_WORKSPACE",
}
F32, F64 = 0, 1
SYMBOL_FD, SYMBOL_SPECTRAL = 0, 1
MULT_SCALE, MULT_HELMHOLTZ, MULT_CN, MULT_EXP, MULT_LAP = 0, 1, 2, 3, 5
MULT_ADV_SOLVE, MULT_ADV_LAP, MULT_ADV_EXP, MULT_TABLE, MULT_ADV_CN = 16, 17, 18, 19, 20
REACT_NONE, REACT_GRAY_SCOTT, REACT_FISHER, REACT_KINETICS = 0, 1, 2, 3
SYMBOL_X_ONLY = 0x10
ETD_1, ETD_2, ETD_RK4 = 1, 2, 4
ETD_COEFF_CONTOUR, ETD_COEFF_PHI = 0, 1


class Grid2DC(C.Structure):
    _fields_ = [("ny", C.c_int), ("nx", C.c_int), ("dy", C.c_double), ("dx", C.c_double)]


class Grid3DC(C.Structure):
    _fields_ = [("nz", C.c_int), ("ny", C.c_int), ("nx", C.c_int), ("pad", C.c_int),
                ("dz", C.c_double), ("dy", C.c_double), ("dx", C.c_double)]


class ETDProblemC(C.Structure):
    _fields_ = [("method", C.c_int), ("coeffs", C.c_int), ("symbol", C.c_int), ("reaction", C.c_int),
                ("nfields", C.c_int), ("pad", C.c_int), ("D", C.c_double * 2), ("F", C.c_double),
                ("k", C.c_double), ("r", C.c_double), ("dt", C.c_double), ("f2_factor", C.c_double)]


class PIDParamsC(C.Structure):
    _fields_ = [(n, C.c_double) for n in
                ("safety", "kI", "kP", "dt_min", "dt_max", "max_factor", "min_factor", "atol", "rtol")]


class ImexProblemC(C.Structure):
    _fields_ = [("reaction", C.c_int), ("nfields", C.c_int), ("D", C.c_double * 4),
                ("F", C.c_double), ("k", C.c_double), ("r", C.c_double), ("dt_cfl", C.c_double),
                ("use_strang", C.c_int), ("max_attempts", C.c_int)]


class NKParamsC(C.Structure):
    _fields_ = [("max_newton_iters", C.c_int), ("max_krylov_iters", C.c_int), ("restart", C.c_int),
                ("max_backtrack", C.c_int), ("newton_tol", C.c_double), ("krylov_tol", C.c_double),
                ("damping", C.c_double), ("backtrack_factor", C.c_double),
                ("min_residual_decrease", C.c_double)]


class ReactorInstanceC(C.Structure):
    _fields_ = [("n", C.c_int), ("variant", C.c_int), ("n_steps", C.c_int), ("pad", C.c_int),
                ("offset", C.c_longlong), ("Pe", C.c_double), ("Da", C.c_double),
                ("dt", C.c_double), ("c_init", C.c_double), ("c_inlet", C.c_double)]


class KineticsC(C.Structure):
    _fields_ = [("nreactions", C.c_int), ("pad", C.c_int), ("order", (C.c_int * 4) * 8),
                ("rate", C.c_double * 8), ("stoich", (C.c_double * 4) * 8), ("linear", (C.c_double * 4) * 4),
                ("source", C.c_double * 4)]


class ExplicitProblemC(C.Structure):
    _fields_ = [("reaction", C.c_int), ("nfields", C.c_int), ("D", C.c_double * 4),
                ("F", C.c_double), ("k", C.c_double), ("r", C.c_double), ("vx", C.c_double),
                ("vy", C.c_double), ("advection", C.c_int), ("method", C.c_int),
                ("bc_kind", C.c_int * 4), ("bc_values", C.c_double * 16), ("dt_cfl", C.c_double),
                ("max_attempts", C.c_int), ("pad", C.c_int), ("kin", KineticsC)]


class AdaptiveResultC(C.Structure):
    _fields_ = [("t_final", C.c_double), ("dt_next", C.c_double), ("prev_err", C.c_double),
                ("last_err", C.c_double), ("n_accepted", C.c_int), ("n_rejected", C.c_int),
                ("n_attempts", C.c_int), ("n_saved", C.c_int), ("status", C.c_int),
                ("finite", C.c_int)]


class GsInstanceC(C.Structure):
    _fields_ = [("ny", C.c_int), ("nx", C.c_int), ("dy", C.c_double), ("dx", C.c_double),
                ("Du", C.c_double), ("Dv", C.c_double), ("F", C.c_double), ("k", C.c_double),
                ("t0", C.c_double), ("t_end", C.c_double), ("dt0", C.c_double), ("dt_cfl", C.c_double),
                ("max_steps", C.c_int), ("save_every", C.c_int), ("max_attempts", C.c_int),
                ("pad", C.c_int), ("pid", PIDParamsC)]


_vp, _sz, _i, _d = C.c_void_p, C.c_size_t, C.c_int, C.c_double
# a linear-operator callback of mjx_gmres_solve: (v, out, user, stream) -> 0 on success
VecOp = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p)

# name -> (restype, argtypes); the list is the exported C ABI
SIGNATURES = {
    "mjx_version": (C.c_char_p, []),
    "mjx_status_string": (C.c_char_p, [_i]),
    "mjx_last_error": (C.c_char_p, []),
    "mjx_spec2d_plan_bytes": (_sz, [_i, _i, _i]),
    "mjx_spec2d_plan_init": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, _vp]),
    "mjx_spec2d_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_spectral_apply2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, C.POINTER(C.c_double), _d, _i,
                                  _vp, _vp, _vp, _sz, _vp]),
    "mjx_advdiff_apply2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_double), _d, _vp, _vp, _vp,
                                 _sz, _vp]),
    "mjx_fft_cn2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _d, _d, _i, _vp, _vp, _vp, _sz, _vp]),
    "mjx_fft_cn2d_noalloc": (_i, [_vp, C.POINTER(Grid2DC), _i, _d, _d, _i, _vp, _vp, _vp]),
    "mjx_gs_cn_ws_bytes": (_sz, [_i, _i, _i]),
    "mjx_gs_strang_exp_ws_bytes": (_sz, [_i, _i, _i]),
    "mjx_gs_rk4_spectral_ws_bytes": (_sz, [_i, _i, _i]),
    "mjx_gs_rk4_spectral2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(C.c_double), _d, _d, _d, _i, _vp, _vp,
                                   _vp, _sz, _vp]),
    "mjx_gs_strang_exp2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(C.c_double), _d, _d, _d, _i, _vp, _vp,
                                 _vp, _sz, _vp]),
    "mjx_gs_cn_newton2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(C.c_double), _d, _d, _d, _i, _d, _i, _vp,
                                _vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double), _vp, _sz, _vp]),
    "mjx_bc_pad2d": (_i, [_vp, _vp, _i, _i, _i, _i, _vp, _vp, _d, _d, _i, _vp]),
    "mjx_bc_fill2d": (_i, [_vp, _vp, _i, _i, _i, _i, _vp, _vp, _d, _d, _i, _vp]),
    "mjx_unpad2d": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp]),
    "mjx_laplacian2d": (_i, [_vp, _vp, _i, _i, _i, _i, _vp, _i, _vp, _vp, _d, _d, _i, _vp]),
    "mjx_stencil1d": (_i, [_vp, _vp, _i, _i, _i, _i, _d, _d, _i, _vp]),
    "mjx_stencil2d": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _i, _d, _d, _i, _vp]),
    "mjx_error_norm_ws_bytes": (_sz, []),
    "mjx_scaled_error_norm": (_i, [_vp, _vp, C.c_longlong, _i, _d, _d, C.POINTER(C.c_double), _vp,
                                   _sz, _vp]),
    "mjx_rhs2d": (_i, [_vp, _vp, _i, _i, _i, _i, _i, _vp, _d, _d, _vp, _vp, _d, _d, _i, _vp]),
    "mjx_imex2d_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_imex_strang_step2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(ImexProblemC), _d,
                                    _vp, _vp, _vp, _sz, _vp]),
    "mjx_imex_adaptive2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(ImexProblemC),
                                 C.POINTER(PIDParamsC), _d, _d, _d, _i, _i, _vp, _vp,
                                 C.POINTER(C.c_double), C.POINTER(C.c_double), _vp, _vp, _sz,
                                 C.POINTER(AdaptiveResultC), _vp]),
    "mjx_reactor_smem_bytes": (_sz, [_i, _i]),
    "mjx_reactor_cn_batch": (_i, [_vp, _i, _i, _i, _vp, _vp]),
    "mjx_reactor_rk4_batch": (_i, [_vp, _i, _i, _i, _vp, _vp]),
    "mjx_gmres_ws_bytes": (_sz, [C.c_longlong, _i]),
    "mjx_gmres_solve": (_i, [C.c_longlong, VecOp, VecOp, _vp, _vp, _vp, _d, _i, _i, C.POINTER(C.c_int),
                             C.POINTER(C.c_double), C.POINTER(C.c_int), _vp, _sz, _vp]),
    "mjx_nk_vardiff_ws_bytes": (_sz, [_i, _i]),
    "mjx_nk_vardiff_integrate2d": (_i, [_vp, _i, _d, _d, C.POINTER(C.c_double), _i, _d, _i, _i,
                                        C.POINTER(NKParamsC), _vp, _vp, C.POINTER(C.c_int), _vp, _sz,
                                        _vp]),
    "mjx_vardiff_rhs2d": (_i, [_i, _d, _d, C.POINTER(C.c_double), _vp, _vp, _vp]),
    "mjx_vardiff_jvp2d": (_i, [_i, _d, _d, C.POINTER(C.c_double), _d, _d, _vp, _vp, _vp, _vp]),
    "mjx_nk_vardiff_step2d": (_i, [_vp, _i, _d, _d, C.POINTER(C.c_double), _i, _d, _d, _i,
                                   C.POINTER(NKParamsC), _vp, _vp, _vp, C.POINTER(C.c_int),
                                   C.POINTER(C.c_double), _vp, _sz, _vp]),
    "mjx_nk_vardiff_adaptive2d": (_i, [_vp, _i, _d, _d, C.POINTER(C.c_double), _i,
                                       C.POINTER(PIDParamsC), _d, _d, _d, _i, _i, _i,
                                       C.POINTER(NKParamsC), _vp, _vp, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double), _vp, C.POINTER(C.c_int),
                                       C.POINTER(C.c_double), _i, C.POINTER(AdaptiveResultC), _vp,
                                       _sz, _vp]),
    "mjx_explicit_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_explicit_integrate2d": (_i, [C.POINTER(Grid2DC), _i, C.POINTER(ExplicitProblemC), _d, _i,
                                      _vp, _vp, _vp, _sz, _vp]),
    "mjx_explicit_rhs2d": (_i, [C.POINTER(Grid2DC), _i, C.POINTER(ExplicitProblemC), _vp, _vp, _vp]),
    "mjx_explicit_adaptive2d": (_i, [C.POINTER(Grid2DC), _i, C.POINTER(ExplicitProblemC),
                                     C.POINTER(PIDParamsC), _d, _d, _d, _i, _i, _vp, _vp,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), _vp, _vp, _sz,
                                     C.POINTER(AdaptiveResultC), _vp]),
    "mjx_dst1_plan_bytes": (_sz, [_i, _i]),
    "mjx_dst1_plan_init": (_i, [_vp, _i, _i, _vp]),
    "mjx_dst1": (_i, [_vp, _i, C.c_longlong, _i, _i, _vp, _vp, _vp, _d, _d, _d, _vp]),
    "mjx_dct2_plan_bytes": (_sz, [_i, _i]),
    "mjx_dct2_plan_init": (_i, [_vp, _i, _i, _vp]),
    "mjx_dct2": (_i, [_vp, _i, C.c_longlong, _i, _i, _vp, _vp, _vp, _d, _d, _d, _vp]),
    "mjx_etdrk4_ws_bytes": (_sz, [_i, _i, _i]),
    "mjx_etdrk4_gray_scott2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, C.POINTER(C.c_double), _d, _d,
                                     _d, _d, _i, _vp, _vp, _vp, _sz, _i, _vp]),
    "mjx_reaction_step2d": (_i, [_vp, _vp, _i, C.c_longlong, _i, _d, _d, _d, _d, _i, _i, _vp]),
    "mjx_variable_diffusion2d": (_i, [_vp, _vp, _i, _vp, _i, _i, _i, _d, _d, _i, _vp]),
    "mjx_advdiff_op2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, C.POINTER(C.c_double), C.POINTER(C.c_double),
                              C.POINTER(C.c_double), _d, _i, _vp, _vp, _vp, _sz, _vp]),
    "mjx_spectral_filter2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, _vp, _vp, _vp, _vp, _sz, _vp]),
    "mjx_dftn_plan_bytes": (_sz, [_i, _i]),
    "mjx_dftn_plan_init": (_i, [_vp, _i, _i, _vp]),
    "mjx_spectral_general2d_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_spectral_apply_general2d": (_i, [_vp, _vp, C.POINTER(Grid2DC), _i, _i, _i, C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.POINTER(C.c_double), _d, _i, _vp, _vp, _vp,
                                          _vp, _sz, _vp]),
    "mjx_spectral_general3d_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_spectral_apply_general3d": (_i, [_vp, _vp, _vp, C.POINTER(Grid3DC), _i, _i, _d, _d, _i, _i, _vp, _vp,
                                          _vp, _sz, _vp]),
    "mjx_spec3d_plan_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_spec3d_plan_init": (_i, [_vp, C.POINTER(Grid3DC), _i, _i, _vp]),
    "mjx_spec3d_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_spectral_apply3d": (_i, [_vp, C.POINTER(Grid3DC), _i, _d, _d, _i, _i, _vp, _vp, _vp, _sz, _vp]),
    "mjx_etd_integrate2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(ETDProblemC), _i, _vp, _vp, _vp, _vp,
                                 _vp, _sz, _i, _vp]),
    "mjx_etd_nonlinear2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _i, _i, _d, _d, _d, _vp, _vp, _vp]),
    "mjx_etdrk4_kernel2d": (_i, [_vp, C.POINTER(Grid2DC), _i, _d, _d, _i, _vp, _sz, _vp]),
    "mjx_imex2d_mixed_ws_bytes": (_sz, [_i, _i, _i]),
    "mjx_imex_adaptive2d_mixed": (_i, [_vp, _vp, C.POINTER(Grid2DC), _i, C.POINTER(ImexProblemC),
                                       C.POINTER(PIDParamsC), _d, _d, _d, _i, _i, _vp, _vp,
                                       C.POINTER(C.c_double), C.POINTER(C.c_double), _vp, _sz,
                                       C.POINTER(AdaptiveResultC), _vp]),
    "mjx_imex_mixed_attempt_kernel2d": (_i, [_vp, _vp, C.POINTER(Grid2DC), C.POINTER(ImexProblemC),
                                             C.POINTER(PIDParamsC), _i, _d, _vp, _vp, _sz, _vp]),
    "mjx_imex_attempt_kernel2d": (_i, [_vp, C.POINTER(Grid2DC), _i, C.POINTER(ImexProblemC),
                                       C.POINTER(PIDParamsC), _i, _d, _vp, _vp, _sz, _vp]),
    "mjx_imex_plan_ws_bytes": (_sz, [_i, _i, _i, _i]),
    "mjx_imex_plan_create": (_i, [C.POINTER(C.c_void_p), _vp, _vp, C.POINTER(Grid2DC), C.POINTER(ImexProblemC),
                                  C.POINTER(PIDParamsC), _i, _i, _vp, _sz]),
    "mjx_imex_plan_run": (_i, [_vp, _i, _d, _d, _d, _vp, _vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                               C.POINTER(AdaptiveResultC), _vp]),
    "mjx_imex_plan_destroy": (_i, [_vp]),
    "mjx_gsbatch_bytes": (_sz, [_i, _i]),
    "mjx_gsbatch_instance_bytes": (_sz, [_i, _i, _i]),
    "mjx_gsbatch_work_items": (_i, [_i, _i]),
    "mjx_gsbatch_create": (_i, [C.POINTER(C.c_void_p), _i, _i, _vp, _sz]),
    "mjx_gsbatch_destroy": (_i, [_vp]),
    "mjx_gsbatch_admit": (_i, [_vp, C.POINTER(GsInstanceC), _i, _vp, _vp, _sz, C.POINTER(C.c_int), _vp]),
    "mjx_gsbatch_run": (_i, [_vp, _i, _i, C.POINTER(C.c_int), C.POINTER(C.c_int), _vp]),
    "mjx_gsbatch_finished": (_i, [_vp, C.POINTER(C.c_int), _i, C.POINTER(C.c_int)]),
    "mjx_gsbatch_retire": (_i, [_vp, _i, _i, _vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                C.POINTER(AdaptiveResultC), _vp]),
    "mjx_gsbatch_request_stop": (None, [_vp, _i]),
    "mjx_dft_schedule_candidates": (_i, [_i, C.POINTER(C.c_int), _i]),
    "mjx_dft_schedule_set": (_i, [_i, _i, _i, C.POINTER(C.c_int), _i]),
    "mjx_dft_schedule_get": (_i, [_i, _i, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mjx_autotune_dft": (_i, [_vp, _i, _i, C.c_longlong, _vp, _sz, _i, C.POINTER(C.c_double), _i,
                              C.POINTER(C.c_int), C.POINTER(C.c_int), _vp]),
    "mjx_stencil_rows_set": (_i, [_i, _i, _i, _i, _i]),
    "mjx_stencil_rows_get": (_i, [_i, _i, _i, _i]),
    "mjx_autotune_stencil2d": (_i, [C.POINTER(Grid2DC), _i, C.POINTER(ExplicitProblemC), _vp, _sz, _i,
                                    C.POINTER(C.c_double), _i, C.POINTER(C.c_int), _vp]),
}


class NativeError(RuntimeError):
    def __init__(self, fn, status):
        msg = f"{fn} failed: {STATUS_NAMES.get(status, status)}"
        if status == 8 and _lib is not None:
            msg += f" [{_lib.mjx_last_error().decode(errors='replace')}]"
        super().__init__(msg)
        self.status = status


def load(path: str | None = None):
    """Loads (once) and returns the native library; raises if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB
        if not os.path.exists(p):
            raise RuntimeError(
                f"native library {p} is missing: run moljax_gb300.build_native.build() "
                "(or __graft_entry__.build()) first")
        lib = C.CDLL(p)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def lib():
    return _lib if _lib is not None else load()


def check(name, status):
    if status != MJX_OK:
        raise NativeError(name, status)


def require_cuda(*tensors):
    if not torch.cuda.is_available():
        raise RuntimeError("moljax_gb300 needs a CUDA GPU: no CPU fallback exists")
    for t in tensors:
        if t is not None and (not t.is_cuda or not t.is_contiguous()):
            raise ValueError("device buffers must be contiguous CUDA tensors")


def dtype_code(dt: torch.dtype) -> int:
    if dt == torch.float32:
        return F32
    if dt == torch.float64:
        return F64
    raise TypeError(f"unsupported dtype {dt}; use float32 or float64")


def stream_ptr(device=None):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)
