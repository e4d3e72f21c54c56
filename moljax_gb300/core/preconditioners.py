"""Preconditioners (moljax/core/preconditioners.py drop-in).

``DiffusionPreconditioner`` accepts both spellings:

* reference form ``DiffusionPreconditioner(field_diffusivities={...},
  n_iterations=5, omega=0.6667)`` -- weighted Jacobi on (I - dt D Lap)
  (preconditioners.py:121-198), applied with torch on padded fields;
* README form ``DiffusionPreconditioner(D, dx, dt)`` (README.md:148) -- the
  exact diagonal inverse (alpha0 I - kappa Lap_D)^-1 for homogeneous Dirichlet
  ghosts by the sine transform (here through the odd extension to a periodic
  box and the native spectral pass).  The native Newton-Krylov driver applies
  the same inverse inside its Arnoldi step as a real DST-II / DST-III pair of
  n-point transforms.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Dict, Optional

import torch


class PrecondContext:
    """preconditioners.py:29-43."""

    def __init__(self, grid, dt, params, **kw):
        self.grid, self.dt, self.params = grid, dt, params
        for k, v in kw.items():
            setattr(self, k, v)


@dataclass(frozen=True)
class IdentityPreconditioner:
    name: str = "identity"

    def apply(self, r, context):
        return r


@dataclass(frozen=True)
class BlockJacobiPreconditioner:
    """preconditioners.py:69-118: r / (1 + dt D 4/dx^2 + dt |v|/dx) per field."""
    name: str = "block_jacobi"
    diffusion_keys: Optional[Dict[str, str]] = None
    advection_keys: Optional[Dict[str, str]] = None

    def apply(self, r, context):
        g, dt, params = context.grid, context.dt, context.params
        out = {}
        for name, f in r.items():
            scale = 1.0
            if self.diffusion_keys and name in self.diffusion_keys:
                scale += dt * params.get(self.diffusion_keys[name], 0.0) * 4.0 / g.min_dx2
            if self.advection_keys and name in self.advection_keys:
                v = params.get(self.advection_keys[name], 0.0)
                scale += dt * float(torch.as_tensor(v).abs().max()) / g.min_dx
            out[name] = f / scale
        return out


class DiffusionPreconditioner:
    """Both spellings; see the module docstring."""

    def __init__(self, D=None, dx=None, dt=None, *, name: str = "diffusion",
                 field_diffusivities: Optional[Dict[str, str]] = None, n_iterations: int = 5,
                 omega: float = 0.6667, alpha0: float = 1.0):
        self.name = name
        self.field_diffusivities = field_diffusivities
        self.n_iterations = n_iterations
        self.omega = omega
        self.spectral = D is not None and not isinstance(D, dict)
        if isinstance(D, dict):
            self.field_diffusivities = D
        self.D, self.dx, self.dt, self.alpha0 = D, dx, dt, alpha0

    # -- reference Jacobi form (preconditioners.py:146-198)
    def _jacobi(self, rhs, grid, dt, D):
        from moljax_gb300.core.stencil import laplacian_2d
        diag = 1.0 + dt * D * (2.0 / grid.dx ** 2 + 2.0 / grid.dy ** 2)
        x = rhs
        for _ in range(self.n_iterations):
            x = self.omega * (rhs + dt * D * laplacian_2d(x, grid)) / diag + (1.0 - self.omega) * x
        return x

    def apply(self, r, context):
        if self.spectral:
            return {k: self.solve(v, context.grid) for k, v in r.items()}
        out = {}
        for name, f in r.items():
            key = (self.field_diffusivities or {}).get(name)
            D = context.params.get(key, 0.0) if key is not None else 0.0
            out[name] = self._jacobi(f, context.grid, context.dt, D) if D > 1e-14 else f
        return out

    def solve(self, r_interior: torch.Tensor, grid=None):
        """(alpha0 I - dt D Lap_D)^-1 r on an interior (n, n) field (Dirichlet ghosts)."""
        n = r_interior.shape[-1]
        dx = float(self.dx if self.dx is not None else grid.dx)
        return dirichlet_helmholtz(r_interior, dx, dx, self.alpha0, float(self.dt) * float(self.D))


def dirichlet_helmholtz(r: torch.Tensor, dy: float, dx: float, alpha: float, kappa: float):
    """(alpha I - kappa Lap_D)^-1 r for homogeneous Dirichlet ghosts (cell-centred).

    The odd extension of r to a (2ny, 2nx) periodic box turns Lap_D into the
    periodic 5-point Laplacian; the native Helmholtz pass inverts it exactly.
    """
    from moljax_gb300.core.fft_solvers import get_plan
    from moljax_gb300 import _native as N
    ny, nx = r.shape[-2:]
    e = torch.empty((2 * ny, 2 * nx), dtype=r.dtype, device=r.device)
    e[:ny, :nx] = r
    e[:ny, nx:] = -r.flip(-1)
    e[ny:, :] = -e[:ny, :].flip(0)
    plan = get_plan(2 * ny, 2 * nx, dy, dx, "fd", r.dtype, r.device)
    out = plan.apply(e, kappa / alpha, 1.0, N.MULT_HELMHOLTZ)
    return out[:ny, :nx] / alpha


def _interior_view(r_field, grid):
    """(interior tensor, is_interior_only) as the reference's shape test
    (preconditioners.py:240-255)."""
    if tuple(r_field.shape) == (grid.ny, grid.nx):
        return r_field, True
    return r_field[grid.interior_slice], False


def _embed(r_field, x_interior, grid, interior_only):
    if interior_only:
        return x_interior
    out = r_field.clone()
    out[grid.interior_slice] = x_interior
    return out


@dataclass(frozen=True)
class FFTDiffusionPreconditioner:
    """Exact periodic (I - dt D Lap)^-1 per diffusive field (preconditioners.py:201-294),
    one native spectral pass per field."""
    name: str = "fft_diffusion"
    field_diffusivity_keys: Optional[Dict[str, str]] = None
    fft_cache: Any = None
    fallback: Optional[Any] = None

    def apply(self, r, context):
        from moljax_gb300.core.fft_solvers import _plan_of
        from moljax_gb300 import _native as N
        if self.fft_cache is None:
            return self.fallback.apply(r, context) if self.fallback is not None else r
        g, dt, params = context.grid, context.dt, context.params
        out = {}
        for name, f in r.items():
            key = (self.field_diffusivity_keys or {}).get(name)
            D = float(params.get(key, 0.0)) if key else 0.0
            if D > 1e-14:
                ri, only = _interior_view(f, g)
                plan = _plan_of(self.fft_cache, g.ny, g.nx, ri.dtype)
                out[name] = _embed(f, plan.apply(ri.contiguous(), D, dt, N.MULT_HELMHOLTZ), g, only)
            else:
                out[name] = f
        return out


@dataclass(frozen=True)
class FFTAdvectionDiffusionPreconditioner:
    """Exact periodic (I - dt(-v.grad + D Lap))^-1 per field (preconditioners.py:297-420):
    FFT2(r) / (1 - dt (D lam - i (vx kx + vy ky))), real part of the inverse, one native pass.
    A field's velocity parameter may be a scalar (vx only) or a (vx, vy) pair."""
    name: str = "fft_advection_diffusion"
    field_diffusivity_keys: Optional[Dict[str, str]] = None
    field_velocity_keys: Optional[Dict[str, str]] = None
    fft_cache: Any = None
    fallback: Optional[Any] = None

    def apply(self, r, context):
        import ctypes as C
        from moljax_gb300.core.fft_solvers import _plan_of, workspace
        from moljax_gb300 import _native as N
        if self.fft_cache is None:
            return self.fallback.apply(r, context) if self.fallback is not None else r
        g, dt, params = context.grid, context.dt, context.params
        out = {}
        for name, f in r.items():
            dkey = (self.field_diffusivity_keys or {}).get(name)
            vkey = (self.field_velocity_keys or {}).get(name)
            D = float(params.get(dkey, 0.0)) if dkey else 0.0
            v = params.get(vkey, 0.0) if vkey else 0.0
            vx, vy = (float(v[0]), float(v[1])) if isinstance(v, (tuple, list)) else (float(v), 0.0)
            if D > 1e-14 or abs(vx) > 1e-14 or abs(vy) > 1e-14:
                ri, only = _interior_view(f, g)
                ri = ri.contiguous()
                N.require_cuda(ri)
                plan = _plan_of(self.fft_cache, g.ny, g.nx, ri.dtype)
                ws = workspace(plan.ws_bytes(1), plan.device)
                x = torch.empty_like(ri)
                N.check("mjx_advdiff_apply2d", N.lib().mjx_advdiff_apply2d(
                    N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, 1, (C.c_double * 1)(D),
                    (C.c_double * 1)(vx), (C.c_double * 1)(vy), float(dt), N.ptr(ri), N.ptr(x),
                    N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
                out[name] = _embed(f, x, g, only)
            else:
                out[name] = f
        return out


def create_gray_scott_preconditioner() -> BlockJacobiPreconditioner:
    """Block-Jacobi on u (Du) and v (Dv) (preconditioners.py:423-427)."""
    return BlockJacobiPreconditioner(diffusion_keys={"u": "Du", "v": "Dv"})


def create_advdiff_preconditioner(field_names) -> BlockJacobiPreconditioner:
    """Block-Jacobi with diffusivity key 'D' and velocity key 'vx' per field
    (preconditioners.py:430-437)."""
    return BlockJacobiPreconditioner(diffusion_keys={n: "D" for n in field_names},
                                     advection_keys={n: "vx" for n in field_names})


def create_diffusion_preconditioner(field_diffusivities: Dict[str, str], n_iterations: int = 5):
    """preconditioners.py:440-457."""
    return DiffusionPreconditioner(field_diffusivities=field_diffusivities, n_iterations=n_iterations)


def create_fft_preconditioner(field_diffusivity_keys: Dict[str, str], fft_cache, fallback=None):
    """preconditioners.py:460-480."""
    return FFTDiffusionPreconditioner(field_diffusivity_keys=field_diffusivity_keys, fft_cache=fft_cache,
                                      fallback=fallback)


def create_gray_scott_fft_preconditioner(fft_cache):
    """FFT preconditioner on u (Du) and v (Dv) (preconditioners.py:483-488)."""
    return FFTDiffusionPreconditioner(field_diffusivity_keys={"u": "Du", "v": "Dv"}, fft_cache=fft_cache)


def create_advdiff_fft_preconditioner(field_diffusivity_keys: Dict[str, str],
                                      field_velocity_keys: Dict[str, str], fft_cache, fallback=None):
    """preconditioners.py:491-514."""
    return FFTAdvectionDiffusionPreconditioner(field_diffusivity_keys=field_diffusivity_keys,
                                               field_velocity_keys=field_velocity_keys,
                                               fft_cache=fft_cache, fallback=fallback)


Preconditioner = Any
