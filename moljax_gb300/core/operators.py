"""Spatial operators (moljax/core/operators.py drop-in).

The operator objects keep the reference's protocol -- ``LinearOp`` /
``NonlinearOp`` with ``apply(state, grid, t, params) -> StateDict``
(operators.py:329-361) -- and additionally carry a ``kind`` that names the
native kernel implementing them, so a model built from them runs fused on the
GPU.  Ops without a kind (user Python callables) still work through
``apply`` but the fused drivers refuse them instead of silently falling back.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Callable, Dict, Optional

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.grid import Grid1D, Grid2D


@dataclass(frozen=True)
class LinearOp:
    name: str
    apply: Callable
    dt_bound: Optional[Callable] = None
    kind: Optional[str] = None


@dataclass(frozen=True)
class NonlinearOp:
    name: str
    apply: Callable
    dt_bound: Optional[Callable] = None
    kind: Optional[int] = None  # native reaction id (MJX_REACT_*)


def laplacian_2d(f, grid: Grid2D):
    """5-point Laplacian on the interior, ghosts zero (operators.py:311-322)."""
    from moljax_gb300.core import stencil
    return stencil.laplacian_2d(f, grid)


def _d1_2d(f, grid: Grid2D, op: int, axis: int, v: float = 0.0):
    from moljax_gb300 import _native as N
    N.require_cuda(f)
    f3 = f.reshape(-1, grid.ny_total, grid.nx_total).contiguous()
    out = torch.empty_like(f3)
    d = grid.dy if axis == 0 else grid.dx
    N.check("mjx_stencil2d", N.lib().mjx_stencil2d(
        N.ptr(f3), N.ptr(out), f3.shape[0], grid.ny, grid.nx, grid.n_ghost, op, axis, float(v),
        float(d), N.dtype_code(f.dtype), N.stream_ptr(f.device)))
    return out.reshape(f.shape)


def d1_upwind_2d(f, v, grid: Grid2D, axis: int):
    """Upwind first derivative along axis (0: y, 1: x) with scalar velocity v, ghosts read as
    stored, result ghosts zero (operators.py:200-268)."""
    if not isinstance(v, (int, float)):
        raise NotImplementedError("d1_upwind_2d: the native stencil takes a scalar velocity")
    return _d1_2d(f, grid, 1, axis, v)


def d1_central_2d(f, grid: Grid2D, axis: int):
    """Central first derivative along axis (operators.py:155-197)."""
    return _d1_2d(f, grid, 2, axis)


def laplacian_1d(f_or_grid, grid=None, order: int = 2):
    """``laplacian_1d(f, grid)`` (operators.py:141-152) or the README factory form
    ``laplacian_1d(grid, order=2)`` returning an operator usable with ``@``."""
    from moljax_gb300.core import stencil1d
    if isinstance(f_or_grid, Grid1D):
        if order != 2:
            raise NotImplementedError("only 2nd-order stencils are built")
        return stencil1d.Operator1D(f_or_grid, "laplacian")
    return stencil1d.laplacian_1d(f_or_grid, grid)


def d1_upwind_1d(f, v, grid: Grid1D):
    """First-order upwind derivative (operators.py:64-110)."""
    from moljax_gb300.core import stencil1d
    return stencil1d.d1_upwind_1d(f, v, grid)


def gradient_1d(grid: Grid1D, upwind: bool = True, v: float = 1.0):
    """README.md:94 factory: ``D1 @ c`` applies d1_upwind_1d with velocity v
    (or the central difference when upwind=False)."""
    from moljax_gb300.core import stencil1d
    return stencil1d.Operator1D(grid, "upwind" if upwind else "central", v=v)


def gray_scott_reaction_op() -> NonlinearOp:
    """u: -uv^2 + F(1-u); v: uv^2 - (F+k)v (operators.py:644-677)."""

    def apply(state, grid, t, params):
        u, v = state["u"], state["v"]
        F, k = params.get("F", 0.04), params.get("k", 0.06)
        uvv = u * v * v
        return {"u": -uvv + F * (1.0 - u), "v": uvv - (F + k) * v}

    def dt_bound(grid, state, params):
        return 0.5 / (params.get("F", 0.04) + params.get("k", 0.06) + 1e-14)

    return NonlinearOp("gray_scott_reaction", apply, dt_bound, N.REACT_GRAY_SCOTT)


def fisher_kpp_reaction_op(field_name: str = "u", r_param: str = "r") -> NonlinearOp:
    """r u (1-u) (operators.py:680-705)."""

    def apply(state, grid, t, params):
        import torch
        out = {k: torch.zeros_like(v) for k, v in state.items()}
        u = state[field_name]
        out[field_name] = params.get(r_param, 1.0) * u * (1.0 - u)
        return out

    def dt_bound(grid, state, params):
        return 0.5 / (params.get(r_param, 1.0) + 1e-14)

    return NonlinearOp(f"fisher_kpp_{field_name}", apply, dt_bound, N.REACT_FISHER)


def fd_laplacian_symbol_2d(ny, nx, dy, dx, dtype=None):
    """operators.py:734-766 (same as fft_solvers.laplacian_symbol_2d)."""
    import torch
    from moljax_gb300.core.fft_solvers import laplacian_symbol_2d
    return laplacian_symbol_2d(ny, nx, dy, dx, dtype or torch.float64)


Params = Dict[str, Any]
