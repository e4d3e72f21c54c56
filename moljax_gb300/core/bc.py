"""Boundary-condition specification (moljax/core/bc.py:26-78).

Ghost cells are filled on the GPU by the native kernels (``apply_bc`` below
calls ``mjx_bc_fill2d``/``mjx_bc_fill1d``); the FFT paths work on interiors
and never materialise ghosts inside their loops.  Values/fluxes are constants
per side (callables are evaluated once on the host at t).
"""

from __future__ import annotations

from dataclasses import dataclass
from enum import IntEnum
from typing import Callable, Dict, Optional


class BCType(IntEnum):
    PERIODIC = 0
    DIRICHLET = 1
    NEUMANN = 2


@dataclass(frozen=True)
class FieldBCSpec:
    kind: BCType
    value: Optional[Callable] = None
    flux: Optional[Callable] = None

    @classmethod
    def periodic(cls) -> "FieldBCSpec":
        return cls(kind=BCType.PERIODIC)

    @classmethod
    def dirichlet(cls, value: Optional[Callable] = None) -> "FieldBCSpec":
        return cls(kind=BCType.DIRICHLET, value=value)

    @classmethod
    def neumann(cls, flux: Optional[Callable] = None) -> "FieldBCSpec":
        return cls(kind=BCType.NEUMANN, flux=flux)


BCSpec = Dict[str, FieldBCSpec]


def side_values(spec: FieldBCSpec, grid, t: float = 0.0, params=None):
    """Per-side constants (left, right, bottom, top) of a field's BC at time t.

    Follows moljax/core/bc.py:173-197 / 322-351: scalars apply to all sides,
    dicts name the sides, anything else means zero.
    """
    fn = spec.value if spec.kind == BCType.DIRICHLET else spec.flux
    if fn is None or spec.kind == BCType.PERIODIC:
        return (0.0, 0.0, 0.0, 0.0)
    params = params or {}
    from moljax_gb300.core.grid import Grid1D
    if isinstance(grid, Grid1D):
        v = fn(grid.x_coords(), t, params)
        try:
            import torch
            v = torch.as_tensor(v, dtype=torch.float64)
            if v.ndim == 0:
                return (float(v), float(v), 0.0, 0.0)
            return (float(v[0]), float(v[-1]), 0.0, 0.0)
        except Exception:  # pragma: no cover - defensive
            return (0.0, 0.0, 0.0, 0.0)
    X, Y = grid.meshgrid()
    v = fn(X, Y, t, params)
    if isinstance(v, dict):
        return tuple(float(v.get(k, 0.0)) for k in ("left", "right", "bottom", "top"))
    import torch
    v = torch.as_tensor(v)
    if v.ndim == 0:
        f = float(v)
        return (f, f, f, f)
    return (0.0, 0.0, 0.0, 0.0)


def create_default_bc_spec(field_names, bc_type: BCType = BCType.PERIODIC) -> BCSpec:
    """moljax/core/bc.py:407-421."""
    return {name: FieldBCSpec(kind=bc_type) for name in field_names}


def apply_bc(state, grid, bc_spec: BCSpec, t: float = 0.0, params=None):
    """Fills ghost cells of every field on the GPU (moljax/core/bc.py:358-404)."""
    from moljax_gb300.core import stencil
    return stencil.apply_bc(state, grid, bc_spec, t, params)
