"""Status codes and small helpers (moljax/core/utils.py)."""

from __future__ import annotations


class StatusCode:
    """moljax/core/utils.py:265-272."""
    SUCCESS = 0
    RUNNING = 1
    MAX_STEPS_REACHED = 2
    DT_TOO_SMALL = 3
    NON_FINITE_VALUES = 4
    NK_FAILED = 5


def get_interior(field, grid):
    """Interior view of a padded field (moljax/core/utils.py:24-40)."""
    return field[grid.interior_slice]


def _interiors(state, grid):
    import torch
    names = list(state.keys())
    return torch.stack([state[n][grid.interior_slice] for n in names]).contiguous()


def scaled_error_norm(err, y_new, grid, atol: float, rtol: float) -> float:
    """sqrt(mean((err / (atol + rtol |y_new|))^2)) over the interiors of every field
    (moljax/core/state.py:312-343), one native reduction kernel."""
    import ctypes as C
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import workspace
    e = _interiors(err, grid)
    y = _interiors(y_new, grid).to(e.dtype)
    N.require_cuda(e)
    ws = workspace(N.lib().mjx_error_norm_ws_bytes(), e.device, "errnorm")
    res = (C.c_double * 2)()
    N.check("mjx_scaled_error_norm", N.lib().mjx_scaled_error_norm(
        N.ptr(e), N.ptr(y), e.numel(), N.dtype_code(e.dtype), float(atol), float(rtol), res,
        N.ptr(ws), ws.numel(), N.stream_ptr(e.device)))
    return float(res[0])


def is_finite(state) -> bool:
    """True when every entry of every field is finite (moljax/core/utils.py:186-197)."""
    import ctypes as C
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import workspace
    for f in state.values():
        t = f.contiguous()
        N.require_cuda(t)
        ws = workspace(N.lib().mjx_error_norm_ws_bytes(), t.device, "errnorm")
        res = (C.c_double * 2)()
        N.check("mjx_scaled_error_norm", N.lib().mjx_scaled_error_norm(
            N.ptr(t), N.ptr(t), t.numel(), N.dtype_code(t.dtype), 1.0, 0.0, res, N.ptr(ws),
            ws.numel(), N.stream_ptr(t.device)))
        if res[1] == 0.0:
            return False
    return True
