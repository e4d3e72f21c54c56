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
    native: Any = None          # the native description (MJX_REACT_KINETICS: (species, KineticsC))


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


def d2_central_2d(f, grid: Grid2D, axis: int):
    """(f[+1] - 2 f + f[-1]) / d^2 along axis (0: y, 1: x) on the interior, ghosts zero
    (operators.py:271-308)."""
    return _d1_2d(f, grid, 3, axis)


def d2_central_1d(f, grid: Grid1D):
    """(f[i+1] - 2 f[i] + f[i-1]) / dx^2 on the interior (operators.py:113-138)."""
    from moljax_gb300.core import stencil1d
    return stencil1d.laplacian_1d(f, grid)


def d1_central_1d(f, grid: Grid1D):
    """(f[i+1] - f[i-1]) / (2 dx) on the interior."""
    from moljax_gb300.core import stencil1d
    return stencil1d.d1_central_1d(f, grid)


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


# ----------------------------------------------------------------- operator factories
def state_zero_like(state):
    """Zeros shaped like each field (operators.py:383-385)."""
    return {k: torch.zeros_like(v) for k, v in state.items()}


def op_sum(ops):
    """(state, grid, t, params) -> the sum of the ops' outputs (operators.py:364-380)."""
    def combined_apply(state, grid, t, params):
        result = ops[0].apply(state, grid, t, params)
        for op in ops[1:]:
            r = op.apply(state, grid, t, params)
            result = {k: result[k] + r[k] for k in result}
        return result
    return combined_apply


def make_diffusion_op_1d(field_name: str, D_param: str = "D") -> LinearOp:
    """D Lap of one field, zeros elsewhere; dt bound 0.5 dx^2 / D (operators.py:392-417)."""
    def apply(state, grid, t, params):
        out = state_zero_like(state)
        out[field_name] = params.get(D_param, 1.0) * laplacian_1d(state[field_name], grid)
        return out

    def dt_bound(grid, params):
        return 0.5 * grid.min_dx2 / (params.get(D_param, 1.0) + 1e-14)

    return LinearOp(f"diffusion_{field_name}", apply, dt_bound, "diffusion")


def make_diffusion_op_2d(field_name: str, D_param: str = "D") -> LinearOp:
    """D Lap of one field, zeros elsewhere; dt bound 0.25 min(dx,dy)^2 / D (operators.py:420-444)."""
    def apply(state, grid, t, params):
        out = state_zero_like(state)
        out[field_name] = params.get(D_param, 1.0) * laplacian_2d(state[field_name], grid)
        return out

    def dt_bound(grid, params):
        return 0.25 * grid.min_dx2 / (params.get(D_param, 1.0) + 1e-14)

    return LinearOp(f"diffusion_{field_name}", apply, dt_bound, "diffusion")


def make_advection_op_1d(field_name: str, vx_param: str = "vx", use_upwind: bool = True) -> LinearOp:
    """-vx df/dx (upwind or central), zeros elsewhere; dt bound dx / |vx| (operators.py:447-481)."""
    def apply(state, grid, t, params):
        vx = params.get(vx_param, 0.0)
        f = state[field_name]
        d = d1_upwind_1d(f, vx, grid) if use_upwind else d1_central_1d(f, grid)
        out = state_zero_like(state)
        out[field_name] = -vx * d
        return out

    def dt_bound(grid, params):
        return grid.min_dx / (abs(params.get(vx_param, 0.0)) + 1e-14)

    return LinearOp(f"advection_{field_name}", apply, dt_bound, "advection")


def make_advection_op_2d(field_name: str, vx_param: str = "vx", vy_param: str = "vy",
                         use_upwind: bool = True) -> LinearOp:
    """-(vx df/dx + vy df/dy), zeros elsewhere; dt bound min(dx,dy) / (|vx| + |vy|)
    (operators.py:484-527)."""
    def apply(state, grid, t, params):
        vx, vy = params.get(vx_param, 0.0), params.get(vy_param, 0.0)
        f = state[field_name]
        if use_upwind:
            dx_, dy_ = d1_upwind_2d(f, vx, grid, 1), d1_upwind_2d(f, vy, grid, 0)
        else:
            dx_, dy_ = d1_central_2d(f, grid, 1), d1_central_2d(f, grid, 0)
        out = state_zero_like(state)
        out[field_name] = -vx * dx_ - vy * dy_
        return out

    def dt_bound(grid, params):
        v = abs(params.get(vx_param, 0.0)) + abs(params.get(vy_param, 0.0))
        return grid.min_dx / (v + 1e-14)

    return LinearOp(f"advection_{field_name}", apply, dt_bound, "advection")


def make_reaction_op(reactions) -> NonlinearOp:
    """Per-field reaction functions (state, params) -> rate, zeros elsewhere
    (operators.py:623-641).  User callables: usable through ``apply`` and the generic
    Newton-Krylov path; the fused drivers take the built-in reactions only."""
    def apply(state, grid, t, params):
        out = state_zero_like(state)
        for name, fn in reactions.items():
            out[name] = fn(state, params)
        return out

    return NonlinearOp("reactions", apply, None, None)


def make_kinetics_op(species, reactions=(), linear=None, source=None) -> NonlinearOp:
    """A mass-action reaction network over the named species (at most 4, the model's
    fields in order, at most 8 reactions) in native form: the multispecies reaction
    terms that make_reaction_op (operators.py:623-641) takes as Python callables, here
    evaluated inside the fused stencil stage kernels (``MJX_REACT_KINETICS``).

    reactions: (rate, reactants, products) with reactants {species: order (1..3)} and
    products {species: count}; rate * prod c^order is the reaction's rate.
    linear: {(target, species): k}, the first-order terms dc_target/dt += k c_species.
    source: {species: s}, zeroth-order feeds.
    ``apply`` evaluates the same rates with torch (the generic paths)."""
    from moljax_gb300 import _native as N
    names = list(species)
    if not 1 <= len(names) <= 4:
        raise ValueError("a native network takes 1 to 4 species")
    reactions = [(float(r), dict(a), dict(b)) for r, a, b in reactions]
    if len(reactions) > 8:
        raise ValueError("a native network takes at most 8 reactions")
    idx = {n: i for i, n in enumerate(names)}
    kin = N.KineticsC()
    kin.nreactions = len(reactions)
    for r, (rate, reac, prod) in enumerate(reactions):
        kin.rate[r] = rate
        for n, o in reac.items():
            if int(o) != o or not 1 <= o <= 3:
                raise ValueError("reactant orders are 1, 2 or 3")
            kin.order[r][idx[n]] = int(o)
            kin.stoich[r][idx[n]] -= float(o)
        for n, c in prod.items():
            kin.stoich[r][idx[n]] += float(c)
    for (t, sname), kv in (linear or {}).items():
        kin.linear[idx[t]][idx[sname]] = float(kv)
    for n, v in (source or {}).items():
        kin.source[idx[n]] = float(v)

    def apply(state, grid, t, params):
        c = [state[n] for n in names]
        out = state_zero_like(state)
        for i, n in enumerate(names):
            acc = torch.zeros_like(c[i]) + kin.source[i]
            for j in range(len(names)):
                if kin.linear[i][j] != 0.0:
                    acc = acc + kin.linear[i][j] * c[j]
            out[n] = acc
        for r in range(kin.nreactions):
            w = kin.rate[r]
            for j in range(len(names)):
                for _ in range(kin.order[r][j]):
                    w = w * c[j]
            for i, n in enumerate(names):
                if kin.stoich[r][i] != 0.0:
                    out[n] = out[n] + kin.stoich[r][i] * w
        return out

    return NonlinearOp("kinetics", apply, None, N.REACT_KINETICS, (names, kin))


def fd_laplacian_symbol_1d(nx: int, dx: float, dtype=None):
    """(2 cos(k dx) - 2) / dx^2, k = 2 pi fftfreq (operators.py:708-731)."""
    from moljax_gb300.core.fft_solvers import laplacian_symbol_1d
    return laplacian_symbol_1d(nx, dx, dtype or torch.float64)
