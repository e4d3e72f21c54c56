"""FFT-diagonalised linear operators (moljax/core/fft_operators.py drop-in).

``DiffusionOperator`` (fft_operators.py:80-176): L = D Lap on a periodic 2D
grid, eigenvalues D * lam_FD.  ``matvec``, ``solve`` and ``exp_matvec`` run the
native spectral pass (forward FFT -> multiplier -> inverse FFT in one fused
column kernel between two row kernels).
"""

from __future__ import annotations

from dataclasses import dataclass, field

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.grid import Grid2D


@dataclass(frozen=True)
class DiffusionOperator:
    grid: Grid2D
    D: float
    dtype: torch.dtype = torch.float64
    name: str = field(default="diffusion", repr=False)

    def __post_init__(self):
        if self.D <= 0:
            raise ValueError(f"Diffusion coefficient D must be > 0, got {self.D}")
        if not isinstance(self.grid, Grid2D):
            raise NotImplementedError("DiffusionOperator is built for 2D periodic grids")

    def _plan(self, dtype=None):
        from moljax_gb300.core.fft_solvers import get_plan
        g = self.grid
        return get_plan(g.ny, g.nx, g.dy, g.dx, "fd", dtype or self.dtype)

    @property
    def eigenvalues(self) -> torch.Tensor:
        """D * lam(kx, ky) (fft_operators.py:114-117)."""
        from moljax_gb300.core.fft_solvers import laplacian_symbol_2d
        g = self.grid
        return self.D * laplacian_symbol_2d(g.ny, g.nx, g.dy, g.dx, self.dtype)

    def solve(self, rhs: torch.Tensor, dt: float) -> torch.Tensor:
        """(I - dt D Lap)^-1 rhs (fft_operators.py:126-140)."""
        return self._plan(rhs.dtype).apply(rhs.contiguous(), self.D, dt, N.MULT_HELMHOLTZ)

    def exp_matvec(self, u: torch.Tensor, dt: float) -> torch.Tensor:
        """exp(dt D Lap) u (fft_operators.py:142-150)."""
        return self._plan(u.dtype).apply(u.contiguous(), self.D, dt, N.MULT_EXP)

    def spectral_bounds(self):
        """(lambda_min, lambda_max) = (-4D(1/dx^2 + 1/dy^2), 0) for the FD symbol."""
        g = self.grid
        return (-4.0 * self.D * (1.0 / g.dx ** 2 + 1.0 / g.dy ** 2), 0.0)
