"""FFT-diagonalised linear operators (moljax/core/fft_operators.py drop-in).

``DiffusionOperator`` (fft_operators.py:80-176): L = D Lap on a periodic 1D or
2D grid, eigenvalues D * lam_FD.  ``AdvectionDiffusionOperator`` (179-260):
L = D Lap - v d/dx, eigenvalues D lam_FD - i v k (k = 2 pi fftfreq); 1D as the
reference, and 2D with v = (vx, vy).  ``matvec``, ``solve`` and ``exp_matvec``
run the native spectral pass (forward FFT -> multiplier -> inverse FFT in one
fused column kernel between two row kernels).  A 1D field is carried as two
identical rows of a (2, n) grid: its y modes are zero up to rounding, so each
row is the 1D result.  ``exact_cfl_dt`` is fft_operators.py:263-296.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Dict, List, NamedTuple, Protocol, Tuple, Union, runtime_checkable

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.grid import Grid1D, Grid2D


@runtime_checkable
class FFTLinearOperator(Protocol):
    """fft_operators.py:42-77: what the ETD integrators and FFT solves need of an operator."""
    name: str
    grid: Union[Grid1D, Grid2D]

    @property
    def eigenvalues(self) -> torch.Tensor: ...

    def matvec(self, u: torch.Tensor) -> torch.Tensor: ...

    def solve(self, rhs: torch.Tensor, dt: float) -> torch.Tensor: ...

    def exp_matvec(self, u: torch.Tensor, dt: float) -> torch.Tensor: ...


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

    def spectral_bounds(self) -> "SpectralBounds":
        """Exact bounds of the FD eigenvalues (fft_operators.py:167-176): rho = max |lam|."""
        lam = self.eigenvalues
        return SpectralBounds(rho=float(lam.abs().max()), re_max=float(lam.max()), im_max=0.0,
                              methods_used={"exact_fft": f"DiffusionOperator(D={self.D})"}, warnings=[])


class SpectralBounds(NamedTuple):
    """The fields of moljax.laplace.spectral_bounds.SpectralBounds used by the FFT operators."""
    rho: float
    re_max: float
    im_max: float
    methods_used: Dict[str, str]
    warnings: List[str]


@dataclass(frozen=True)
class AdvectionDiffusionOperator:
    """L u = D Lap u - v . grad u on a periodic grid (fft_operators.py:179-260).

    ``v`` is a float on a Grid1D (the reference form) or (vx, vy) on a Grid2D.
    """
    grid: Union[Grid1D, Grid2D]
    v: Union[float, Tuple[float, float]]
    D: float = 0.0
    dtype: torch.dtype = torch.float64
    name: str = field(default="advection_diffusion", repr=False)

    def __post_init__(self):
        if isinstance(self.grid, Grid1D):
            if not isinstance(self.v, (int, float)):
                raise TypeError("on a Grid1D, v is a float")
        elif not isinstance(self.grid, Grid2D):
            raise TypeError("AdvectionDiffusionOperator takes a Grid1D or Grid2D")

    @property
    def is_1d(self) -> bool:
        return isinstance(self.grid, Grid1D)

    def _velocity(self):
        if self.is_1d:
            return float(self.v), 0.0
        vx, vy = self.v
        return float(vx), float(vy)

    @property
    def eigenvalues(self) -> torch.Tensor:
        """-i v k + D (2 cos(k dx) - 2)/dx^2 (fft_operators.py:223-228), complex, numpy order."""
        from moljax_gb300.core.fft_solvers import (build_wavenumbers_1d, build_wavenumbers_2d,
                                                   laplacian_symbol_1d, laplacian_symbol_2d)
        g = self.grid
        vx, vy = self._velocity()
        if self.is_1d:
            k = build_wavenumbers_1d(g.nx, g.dx, torch.float64)
            lam = laplacian_symbol_1d(g.nx, g.dx, torch.float64)
            adv = -1j * vx * k
        else:
            kx, ky = build_wavenumbers_2d(g.ny, g.nx, g.dy, g.dx, torch.float64)
            lam = laplacian_symbol_2d(g.ny, g.nx, g.dy, g.dx, torch.float64).cpu()
            adv = -1j * (vx * kx + vy * ky)
        return (adv + (self.D * lam if self.D > 0 else 0.0)).to(
            torch.complex64 if self.dtype == torch.float32 else torch.complex128)

    def _apply(self, u: torch.Tensor, h: float, op: int) -> torch.Tensor:
        from moljax_gb300.core.fft_solvers import get_plan, workspace
        u = u.contiguous()
        N.require_cuda(u)
        g = self.grid
        if self.is_1d:
            if u.ndim != 1:
                raise ValueError("1D operator: field of shape (nx,)")
            plan = get_plan(2, g.nx, g.dx, g.dx, "fd", u.dtype, u.device)
            x = torch.stack([u, u])
        else:
            plan = get_plan(g.ny, g.nx, g.dy, g.dx, "fd", u.dtype, u.device)
            x = u
        vx, vy = self._velocity()
        if getattr(plan, "general", False):
            mult = (N.MULT_ADV_SOLVE, N.MULT_ADV_LAP, N.MULT_ADV_EXP)[op]
            out = plan.apply(x, float(self.D), h, mult, vx=vx, vy=vy)
            return out[0].clone() if self.is_1d else out
        out = torch.empty_like(x)
        ws = workspace(plan.ws_bytes(1), plan.device)
        D_ = (C.c_double * 1)(float(self.D))
        vx_ = (C.c_double * 1)(vx)
        vy_ = (C.c_double * 1)(vy)
        N.check("mjx_advdiff_op2d", N.lib().mjx_advdiff_op2d(
            N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, 1, D_, vx_, vy_, float(h), int(op),
            N.ptr(x), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
        return out[0].clone() if self.is_1d else out

    def matvec(self, u: torch.Tensor) -> torch.Tensor:
        """real(ifft(lam fft(u))) (fft_operators.py:230-234)."""
        return self._apply(u, 1.0, 1)

    def solve(self, rhs: torch.Tensor, dt: float) -> torch.Tensor:
        """(I - dt L)^-1 rhs, |denominator| clamped at 1e-14 (fft_operators.py:236-242)."""
        return self._apply(rhs, dt, 0)

    def exp_matvec(self, u: torch.Tensor, dt: float) -> torch.Tensor:
        """real(ifft(exp(dt lam) fft(u))) (fft_operators.py:244-249)."""
        return self._apply(u, dt, 2)

    def spectral_bounds(self) -> SpectralBounds:
        """fft_operators.py:251-260."""
        lam = self.eigenvalues.to(torch.complex128)
        return SpectralBounds(rho=float(lam.abs().max()), re_max=float(lam.real.max()),
                              im_max=float(lam.imag.abs().max()),
                              methods_used={"exact_fft": f"AdvectionDiffusionOperator(v={self.v}, D={self.D})"},
                              warnings=[])


def exact_cfl_dt(op, method: str = "explicit", safety: float = 0.9) -> float:
    """fft_operators.py:263-296: explicit safety * 2 / max|lam| (inf when ~0); IMEX and ETD
    safety * 1."""
    if method == "explicit":
        rho = float(op.eigenvalues.abs().max())
        if rho < 1e-14:
            return float("inf")
        return safety * 2.0 / rho
    if method in ("imex", "etd"):
        return safety * 1.0
    raise ValueError(f"Unknown method: {method}")
