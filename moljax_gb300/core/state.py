"""StateDict helpers (moljax/core/state.py drop-in).

A state is a dict of field name -> padded CUDA tensor.  The tree helpers are
elementwise plumbing on those tensors; ``scaled_error_norm`` and ``is_finite``
are the native reductions (``moljax_gb300.core.utils``).
"""

from __future__ import annotations

from typing import Callable, Dict, Tuple

import torch

from moljax_gb300.core.grid import Grid1D
from moljax_gb300.core.utils import is_finite, scaled_error_norm  # noqa: F401  (state.py:312-343)

StateDict = Dict[str, torch.Tensor]


def tree_add(a: StateDict, b: StateDict) -> StateDict:
    """state.py:27-38."""
    return {k: a[k] + b[k] for k in a}


def tree_sub(a: StateDict, b: StateDict) -> StateDict:
    """state.py:41-52."""
    return {k: a[k] - b[k] for k in a}


def tree_scale(a: StateDict, c: float) -> StateDict:
    """state.py:55-66."""
    return {k: c * v for k, v in a.items()}


def tree_axpy(y: StateDict, a: float, x: StateDict) -> StateDict:
    """y + a x (state.py:69-81)."""
    return {k: y[k] + a * x[k] for k in y}


def tree_zeros_like(state: StateDict) -> StateDict:
    return {k: torch.zeros_like(v) for k, v in state.items()}


def tree_ones_like(state: StateDict) -> StateDict:
    return {k: torch.ones_like(v) for k, v in state.items()}


def _interior(field: torch.Tensor, grid) -> torch.Tensor:
    return field[grid.interior_slice]


def tree_norm2(state: StateDict, grid, interior_only: bool = True) -> torch.Tensor:
    """sqrt of the sum of squares over all fields (state.py:115-137)."""
    tot = sum(((_interior(f, grid) if interior_only else f).double() ** 2).sum() for f in state.values())
    return torch.sqrt(tot)


def tree_norm_inf(state: StateDict, grid, interior_only: bool = True) -> torch.Tensor:
    """max |f| over all fields (state.py:140-161)."""
    return torch.stack([(_interior(f, grid) if interior_only else f).abs().max() for f in state.values()]).max()


def tree_vdot(a: StateDict, b: StateDict, grid, interior_only: bool = True) -> torch.Tensor:
    """sum of a * b over all fields (state.py:164-189)."""
    def pick(f):
        return _interior(f, grid) if interior_only else f
    return sum((pick(a[k]).double() * pick(b[k]).double()).sum() for k in a)


def flatten_to_vec(state: StateDict) -> Tuple[torch.Tensor, Callable[[torch.Tensor], StateDict]]:
    """(flat vector in key order, unravel function) (state.py:192-217)."""
    keys = list(state.keys())
    shapes = [state[k].shape for k in keys]
    flat = torch.cat([state[k].reshape(-1) for k in keys])

    def unravel(vec: torch.Tensor) -> StateDict:
        out, o = {}, 0
        for k, s in zip(keys, shapes):
            n = 1
            for d in s:
                n *= d
            out[k] = vec[o:o + n].reshape(s)
            o += n
        return out
    return flat, unravel


def unflatten_from_vec(flat_vec: torch.Tensor, template_state: StateDict) -> StateDict:
    """state.py:220-238."""
    return flatten_to_vec(template_state)[1](flat_vec)


def state_total_size(state: StateDict) -> int:
    return sum(f.numel() for f in state.values())


def state_interior_size(state: StateDict, grid) -> int:
    return sum(_interior(f, grid).numel() for f in state.values())


def create_state_from_interior(interior_arrays: Dict[str, torch.Tensor], grid,
                               dtype=torch.float64) -> StateDict:
    """Zero-padded fields holding the given interiors (state.py:268-295)."""
    out = {}
    for name, a in interior_arrays.items():
        a = torch.as_tensor(a)
        shape = (grid.nx_total,) if isinstance(grid, Grid1D) else (grid.ny_total, grid.nx_total)
        p = torch.zeros(shape, dtype=dtype, device=a.device)
        p[grid.interior_slice] = a.to(dtype)
        out[name] = p
    return out


def get_interior_state(state: StateDict, grid) -> StateDict:
    """state.py:298-309."""
    return {k: _interior(v, grid) for k, v in state.items()}
