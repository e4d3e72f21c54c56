"""FFT-diagonalised linear operators (moljax/core/fft_operators.py drop-in).

``DiffusionOperator`` (fft_operators.py:80-176): L = D Lap on a periodic 1D or
2D grid, eigenvalues D * lam_FD.  ``matvec``, ``solve`` and ``exp_matvec`` run
the native spectral pass (forward FFT -> multiplier -> inverse FFT in one fused
column kernel between two row kernels).  A 1D field is carried as two identical
rows of a (2, n) grid: its y modes are zero up to rounding, so each row is the
1D result.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Union

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.grid import Grid1D, Grid2D


@dataclass(frozen=True)
class DiffusionOperator:
    grid: Union[Grid1D, Grid2D]
    D: float
    dtype: torch.dtype = torch.float64
    name: str = field(default="diffusion", repr=False)

    def __post_init__(self):
        if self.D <= 0:
            raise ValueError(f"Diffusion coefficient D must be > 0, got {self.D}")
        if not isinstance(self.grid, (Grid1D, Grid2D)):
            raise TypeError("DiffusionOperator takes a Grid1D or Grid2D")

    @property
    def is_1d(self) -> bool:
        return isinstance(self.grid, Grid1D)

    def _plan(self, dtype=None):
        from moljax_gb300.core.fft_solvers import get_plan
        g = self.grid
        if self.is_1d:
            return get_plan(2, g.nx, g.dx, g.dx, "fd", dtype or self.dtype)
        return get_plan(g.ny, g.nx, g.dy, g.dx, "fd", dtype or self.dtype)

    @property
    def eigenvalues(self) -> torch.Tensor:
        """D * lam(k) (fft_operators.py:114-117), numpy FFT order."""
        from moljax_gb300.core.fft_solvers import laplacian_symbol_1d, laplacian_symbol_2d
        g = self.grid
        if self.is_1d:
            return self.D * laplacian_symbol_1d(g.nx, g.dx, self.dtype)
        return self.D * laplacian_symbol_2d(g.ny, g.nx, g.dy, g.dx, self.dtype)

    def _apply(self, u: torch.Tensor, h: float, mult: int) -> torch.Tensor:
        u = u.contiguous()
        plan = self._plan(u.dtype)
        if self.is_1d:
            if u.ndim != 1:
                raise ValueError("1D operator: field of shape (nx,)")
            return plan.apply(torch.stack([u, u]), self.D, h, mult)[0].clone()
        return plan.apply(u, self.D, h, mult)

    def matvec(self, u: torch.Tensor) -> torch.Tensor:
        """D Lap u via FFT (fft_operators.py:119-129)."""
        return self._apply(u, 1.0, N.MULT_LAP)

    def solve(self, rhs: torch.Tensor, dt: float) -> torch.Tensor:
        """(I - dt D Lap)^-1 rhs (fft_operators.py:131-149)."""
        return self._apply(rhs, dt, N.MULT_HELMHOLTZ)

    def exp_matvec(self, u: torch.Tensor, dt: float) -> torch.Tensor:
        """exp(dt D Lap) u (fft_operators.py:151-165)."""
        return self._apply(u, dt, N.MULT_EXP)

    def spectral_bounds(self):
        """(lambda_min, lambda_max) = (-4D sum 1/d^2, 0) for the FD symbol."""
        g = self.grid
        if self.is_1d:
            return (-4.0 * self.D / g.dx ** 2, 0.0)
        return (-4.0 * self.D * (1.0 / g.dx ** 2 + 1.0 / g.dy ** 2), 0.0)
