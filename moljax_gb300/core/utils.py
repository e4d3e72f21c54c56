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


# ---------------------------------------------------------------- small helpers (utils.py:20-261)
def eps_for_dtype(dtype=None) -> float:
    """1e-10 for FP32, else 1e-14 (utils.py:20-27)."""
    import torch
    return 1e-10 if dtype == torch.float32 else 1e-14


def safe_eps(dtype=None) -> float:
    return eps_for_dtype(dtype)


def set_interior(padded, interior, grid):
    """A copy of padded with its interior replaced (utils.py:44-60)."""
    out = padded.clone()
    out[grid.interior_slice] = interior
    return out


def allocate_scalar_history(max_steps: int, dtype=None, device=None):
    import torch
    return torch.zeros(max_steps, dtype=dtype or torch.float64, device=device)


def allocate_field_history(field_shape, max_steps: int, dtype=None, device=None):
    import torch
    return torch.zeros((max_steps,) + tuple(field_shape), dtype=dtype or torch.float64, device=device)


def allocate_state_history(state, grid, max_steps: int, interior_only: bool = True, dtype=None):
    """utils.py:96-123."""
    return {n: allocate_field_history((f[grid.interior_slice] if interior_only else f).shape, max_steps,
                                      dtype or f.dtype, f.device) for n, f in state.items()}


def save_to_history(history, state, grid, idx: int, interior_only: bool = True):
    """Writes the state into slot idx (in place) and returns the history (utils.py:126-153)."""
    for n, f in state.items():
        history[n][idx] = f[grid.interior_slice] if interior_only else f
    return history


def safe_divide(numerator, denominator, eps: float = 1e-14):
    return numerator / (denominator + eps)


def clip_array(x, x_min: float, x_max: float):
    import torch
    return torch.clamp(x, x_min, x_max)


def create_padded_array(grid, fill_value: float = 0.0, dtype=None, device=None):
    """utils.py:200-219."""
    import torch
    from moljax_gb300.core.grid import Grid1D
    shape = (grid.nx_total,) if isinstance(grid, Grid1D) else (grid.ny_total, grid.nx_total)
    return torch.full(shape, fill_value, dtype=dtype or torch.float64, device=device)


def max_abs_interior(field, grid):
    return field[grid.interior_slice].abs().max()


def mean_interior(field, grid):
    return field[grid.interior_slice].mean()


def sum_interior(field, grid):
    return field[grid.interior_slice].sum()
