"""1D finite-difference operators on padded fields (native kernels).

``laplacian_1d(f, grid)`` / ``d1_upwind_1d(f, v, grid)`` / ``d1_central_1d``
keep the reference signatures (moljax/core/operators.py:35-152);
``Operator1D`` is the README operator form (README.md:92-95): ``D2 @ c`` and
``D1 @ c`` with ``D2 = laplacian_1d(grid)``, ``D1 = gradient_1d(grid)``.
Applied to an interior vector (length nx) the operator pads it with the
grid's boundary treatment first: Neumann zero-gradient ghosts by default, or
for ``bc_type='danckwerts'`` the Danckwerts inlet (ghost so that the upwind
flux is -(c0 - 1)/dx) and a zero-gradient outlet.
"""

from __future__ import annotations

import torch

from moljax_gb300 import _native as N


def _run(f, grid, op, v=0.0):
    x = f.reshape(-1, f.shape[-1]).contiguous()
    N.require_cuda(x)
    out = torch.empty_like(x)
    N.check("mjx_stencil1d", N.lib().mjx_stencil1d(
        N.ptr(x), N.ptr(out), x.shape[0], grid.nx, grid.n_ghost, op, float(v), grid.dx,
        N.dtype_code(x.dtype), N.stream_ptr(x.device)))
    return out.reshape(f.shape)


def laplacian_1d(f, grid):
    """operators.py:141-152."""
    return _run(f, grid, 0)


def d1_upwind_1d(f, v, grid):
    """operators.py:64-110 (scalar velocity)."""
    if torch.is_tensor(v) and v.ndim > 0:
        raise NotImplementedError("d1_upwind_1d: array velocity is not built (scalar v only)")
    return _run(f, grid, 1, float(v))


def d1_central_1d(f, grid):
    """operators.py:35-61."""
    return _run(f, grid, 2)


class Operator1D:
    """README-form operator: ``op @ c`` on an interior (nx,) or padded (nx+2g,) vector."""

    def __init__(self, grid, kind: str, v: float = 1.0):
        self.grid, self.kind, self.v = grid, kind, v

    def _pad(self, c):
        g = self.grid
        if c.shape[-1] == g.nx_total:
            return c
        ng = g.n_ghost
        p = torch.empty(c.shape[:-1] + (g.nx_total,), dtype=c.dtype, device=c.device)
        p[..., ng:ng + g.nx] = c
        p[..., ng + g.nx:] = c[..., -1:]   # zero-gradient outlet
        if (g.bc_type or "").lower() == "danckwerts" and self.kind == "upwind":
            p[..., :ng] = 1.0 - 0.0 * c[..., :1]  # inflow ghost: upwind flux -(c0 - 1)/dx
        elif (g.bc_type or "").lower() == "danckwerts":
            p[..., :ng] = 0.0 * c[..., :1]        # benchmark_reactor_vs_diffrax.py:40-48 row 0
        else:
            p[..., :ng] = c[..., :1]
        return p

    def __matmul__(self, c):
        g = self.grid
        interior = c.shape[-1] == g.nx
        p = self._pad(c)
        op = {"laplacian": 0, "upwind": 1, "central": 2}[self.kind]
        r = _run(p, g, op, self.v)
        return r[..., g.n_ghost:g.n_ghost + g.nx] if interior else r
