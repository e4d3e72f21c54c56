"""FFT-based solvers on periodic 2D grids (moljax/core/fft_solvers.py drop-in).

All transforms run in the native library: a shared-memory Stockham FFT in
fused row (r2c/c2r) and column (forward * multiplier * inverse) passes.  A
``SpectralPlan`` owns the device tables (twiddles for nx and ny, the 1D
Laplacian symbols); workspaces are caller-side torch buffers, so the step
calls allocate nothing in the native code.

Public names follow the reference: ``laplacian_symbol_2d``,
``create_fft_cache``, ``solve_helmholtz_2d``, ``apply_diffusion_inverse_fft``;
plus the README's ``fft_cn_step(u0, D, dx, dt)`` (README.md:49-58), whose
reference form is benchmark code (benchmarks/benchmark_vs_scipy.py:74-91).
"""

from __future__ import annotations

import ctypes as C
import math
import threading
from typing import Dict, NamedTuple, Optional

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.grid import Grid1D, Grid2D

_plans: Dict[tuple, "SpectralPlan"] = {}
_ws: Dict[tuple, torch.Tensor] = {}

SYMBOLS = {"fd": N.SYMBOL_FD, "spectral": N.SYMBOL_SPECTRAL}


def _device(device=None):
    if device is None:
        return torch.device("cuda", torch.cuda.current_device())
    d = torch.device(device)
    return torch.device("cuda", d.index if d.index is not None else torch.cuda.current_device())


def workspace(nbytes: int, device, tag: str = "ws") -> torch.Tensor:
    """Reusable device scratch of at least nbytes (one per device, tag and host thread,
    so that concurrent solves on per-thread streams never share scratch)."""
    key = (str(device), tag, threading.get_ident())
    buf = _ws.get(key)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)
        _ws[key] = buf
    return buf


class SpectralPlan:
    """Device twiddle and symbol tables for one periodic (ny, nx) grid."""

    def __init__(self, ny: int, nx: int, dy: float, dx: float, symbol: str = "fd",
                 dtype: torch.dtype = torch.float64, device=None):
        N.require_cuda()
        self.ny, self.nx, self.dy, self.dx = int(ny), int(nx), float(dy), float(dx)
        self.symbol = symbol
        self.dtype = dtype
        self.device = _device(device)
        self.code = N.dtype_code(dtype)
        lib = N.lib()
        nbytes = lib.mjx_spec2d_plan_bytes(self.ny, self.nx, self.code)
        if nbytes == 0:
            raise ValueError(f"unsupported grid {ny}x{nx}: sizes must be powers of two in [2, 4096]")
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.cgrid = N.Grid2DC(self.ny, self.nx, self.dy, self.dx)
        with torch.cuda.device(self.device):
            N.check("mjx_spec2d_plan_init", lib.mjx_spec2d_plan_init(
                N.ptr(self.buf), C.byref(self.cgrid), SYMBOLS[symbol], self.code,
                N.stream_ptr(self.device)))

    def ws_bytes(self, nfields: int) -> int:
        return N.lib().mjx_spec2d_ws_bytes(self.ny, self.nx, nfields, self.code)

    def apply(self, x: torch.Tensor, D, h: float, mult: int, out: Optional[torch.Tensor] = None):
        """out_f = IFFT2(m(h, D_f) FFT2(x_f)) for x of shape (ny, nx) or (nf, ny, nx)."""
        x3 = x.reshape(-1, self.ny, self.nx)
        N.require_cuda(x3)
        if x3.dtype != self.dtype:
            raise TypeError(f"plan dtype {self.dtype} does not match {x3.dtype}")
        nf = x3.shape[0]
        Ds = [float(D)] * nf if not isinstance(D, (list, tuple)) else [float(d) for d in D]
        out3 = torch.empty_like(x3) if out is None else out.reshape(-1, self.ny, self.nx)
        Dc = (C.c_double * nf)(*Ds)
        # fields are processed four at a time (the C ABI limit per call)
        for i in range(0, nf, 4):
            j = min(nf, i + 4)
            ws = workspace(self.ws_bytes(j - i), self.device)
            Dcc = (C.c_double * (j - i))(*Ds[i:j])
            N.check("mjx_spectral_apply2d", N.lib().mjx_spectral_apply2d(
                N.ptr(self.buf), C.byref(self.cgrid), self.code, j - i, Dcc, float(h), int(mult),
                N.ptr(x3[i:j]), N.ptr(out3[i:j]), N.ptr(ws), ws.numel(),
                N.stream_ptr(self.device)))
        del Dc
        return out3.reshape(x.shape)


def get_plan(ny, nx, dy, dx, symbol="fd", dtype=torch.float64, device=None) -> SpectralPlan:
    dev = _device(device)
    key = (int(ny), int(nx), float(dy), float(dx), symbol, dtype, str(dev))
    p = _plans.get(key)
    if p is None:
        p = SpectralPlan(ny, nx, dy, dx, symbol, dtype, dev)
        _plans[key] = p
    return p


# ----------------------------------------------------------------- symbols
def build_wavenumbers_1d(nx: int, dx: float, dtype=torch.float64):
    """moljax/core/fft_solvers.py:49-64: k = 2 pi fftfreq(nx, dx)."""
    return (2.0 * math.pi * torch.fft.fftfreq(nx, d=dx, dtype=torch.float64)).to(dtype)


def laplacian_symbol_1d(nx: int, dx: float, dtype=torch.float64):
    """moljax/core/fft_solvers.py:97-121."""
    k = build_wavenumbers_1d(nx, dx)
    return ((2.0 * torch.cos(k * dx) - 2.0) / (dx * dx)).to(dtype)


def laplacian_symbol_2d(ny: int, nx: int, dy: float, dx: float, dtype=torch.float64,
                        device=None):
    """moljax/core/fft_solvers.py:124-154 on the GPU; the tensor carries its plan.

    ``solve_helmholtz_2d`` recognises the attached plan and runs the native
    spectral pass with the separable symbol it encodes.
    """
    lam = (laplacian_symbol_1d(nx, dx)[None, :] + laplacian_symbol_1d(ny, dy)[:, None]).to(dtype)
    dev = _device(device)
    lam = lam.to(dev)
    lam._mjx_plan = get_plan(ny, nx, dy, dx, "fd", dtype, dev)
    return lam


class FFTCache2D(NamedTuple):
    """moljax/core/fft_solvers.py:38-42 plus the native plan."""
    laplacian_symbol: torch.Tensor
    kx: torch.Tensor
    ky: torch.Tensor
    plan: SpectralPlan


def create_fft_cache_2d(grid: Grid2D, dtype=torch.float64, device=None) -> FFTCache2D:
    """moljax/core/fft_solvers.py:181-198."""
    dev = _device(device)
    lam = laplacian_symbol_2d(grid.ny, grid.nx, grid.dy, grid.dx, dtype, dev)
    kx1 = build_wavenumbers_1d(grid.nx, grid.dx, dtype)
    ky1 = build_wavenumbers_1d(grid.ny, grid.dy, dtype)
    kx = kx1[None, :].expand(grid.ny, grid.nx).to(dev)
    ky = ky1[:, None].expand(grid.ny, grid.nx).to(dev)
    return FFTCache2D(lam, kx, ky, lam._mjx_plan)


def create_fft_cache(grid, dtype=torch.float64, device=None):
    """moljax/core/fft_solvers.py:201-215 (2D grids)."""
    if isinstance(grid, Grid1D):
        raise NotImplementedError("1D periodic FFT cache: use Grid2D (1D spectral path not built)")
    return create_fft_cache_2d(grid, dtype, device)


def _plan_of(laplacian_symbol_or_cache, ny, nx, dtype):
    obj = laplacian_symbol_or_cache
    plan = getattr(obj, "plan", None) or getattr(obj, "_mjx_plan", None)
    if plan is None:
        raise NotImplementedError(
            "solve_helmholtz_2d needs a symbol made by laplacian_symbol_2d/create_fft_cache "
            "(the native pass uses the separable FD symbol of that plan)")
    if (plan.ny, plan.nx) != (ny, nx):
        raise ValueError("symbol/grid shape mismatch")
    if plan.dtype != dtype:
        plan = get_plan(plan.ny, plan.nx, plan.dy, plan.dx, plan.symbol, dtype, plan.device)
    return plan


def solve_helmholtz_2d(rhs_interior: torch.Tensor, laplacian_symbol, dt: float, D: float):
    """(I - dt D Lap) u = rhs on the interior (moljax/core/fft_solvers.py:261-294)."""
    ny, nx = rhs_interior.shape[-2:]
    plan = _plan_of(laplacian_symbol, ny, nx, rhs_interior.dtype)
    return plan.apply(rhs_interior.contiguous(), D, dt, N.MULT_HELMHOLTZ)


def solve_helmholtz(rhs_interior, laplacian_symbol, dt, D):
    """moljax/core/fft_solvers.py:297-320 (2D)."""
    if rhs_interior.ndim != 2:
        raise NotImplementedError("1D Helmholtz: use a 2D grid")
    return solve_helmholtz_2d(rhs_interior, laplacian_symbol, dt, D)


def extract_interior(f_padded, grid):
    """moljax/core/fft_solvers.py:327-342."""
    return f_padded[grid.interior_slice]


def embed_interior(u_interior, grid, padded_template):
    """moljax/core/fft_solvers.py:345-365 (ghosts from the template)."""
    out = padded_template.clone()
    out[grid.interior_slice] = u_interior
    return out


def apply_diffusion_inverse_fft(state_rhs, grid: Grid2D, dt: float, diffusivities, fft_cache):
    """(I - dt D Lap)^-1 per diffusive field, ghosts kept (fft_solvers.py:406-445)."""
    from moljax_gb300.core import stencil
    names = [n for n in state_rhs if diffusivities.get(n, 0.0) > 1e-14]
    out = dict(state_rhs)
    if not names:
        return out
    padded = stencil.stack(state_rhs, names)
    interior = stencil.unpad(padded, grid)
    plan = _plan_of(fft_cache, grid.ny, grid.nx, interior.dtype)
    res = plan.apply(interior, [diffusivities[n] for n in names], dt, N.MULT_HELMHOLTZ)
    for i, n in enumerate(names):
        out[n] = embed_interior(res[i], grid, state_rhs[n])
    return out


def fft_cn_step(u0: torch.Tensor, D: float, dx: float, dt: float, n_steps: int = 1,
                symbol: str = "spectral", dy: Optional[float] = None) -> torch.Tensor:
    """Crank-Nicolson steps u <- real(IFFT2(G FFT2(u))), G = (1+dt D lam/2)/(1-dt D lam/2).

    README.md:49-58 name; the reference computes it in the benchmark scripts
    (benchmarks/benchmark_vs_scipy.py:74-91, pseudo-spectral symbol -k^2, the
    default here; ``symbol='fd'`` uses the 5-point symbol).  ``n_steps`` steps
    run one after another on the GPU (each one a full forward/multiply/inverse).
    """
    u = u0.contiguous()
    N.require_cuda(u)
    ny, nx = u.shape[-2:]
    dy = dx if dy is None else dy
    plan = get_plan(ny, nx, dy, dx, symbol, u.dtype, u.device)
    out = torch.empty_like(u)
    ws = workspace(plan.ws_bytes(1), plan.device)
    N.check("mjx_fft_cn2d", N.lib().mjx_fft_cn2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, float(D), float(dt), int(n_steps),
        N.ptr(u), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out


# ----------------------------------------------------------------- periodic 3D boxes
class SpectralPlan3D:
    """Device tables of one periodic [nz][ny][nx] box (benchmarks/sisc/bench_3d_feasibility.py)."""

    def __init__(self, nz: int, ny: int, nx: int, dz: float, dy: float, dx: float,
                 symbol: str = "spectral", dtype: torch.dtype = torch.float64, device=None):
        N.require_cuda()
        self.shape = (int(nz), int(ny), int(nx))
        self.symbol, self.dtype, self.device = symbol, dtype, _device(device)
        self.code = N.dtype_code(dtype)
        lib = N.lib()
        nbytes = lib.mjx_spec3d_plan_bytes(*self.shape, self.code)
        if nbytes == 0:
            raise ValueError(f"unsupported box {nz}x{ny}x{nx}: sizes must be powers of two in [2, 4096]")
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self.cgrid = N.Grid3DC(int(nz), int(ny), int(nx), 0, float(dz), float(dy), float(dx))
        with torch.cuda.device(self.device):
            N.check("mjx_spec3d_plan_init", lib.mjx_spec3d_plan_init(
                N.ptr(self.buf), C.byref(self.cgrid), SYMBOLS[symbol], self.code, N.stream_ptr(self.device)))

    def apply(self, u: torch.Tensor, D: float, h: float, mult: int, n_steps: int = 1) -> torch.Tensor:
        """n_steps times u <- real(IFFTN(m(h, D, lam) FFTN(u))) on the GPU."""
        u = u.contiguous()
        N.require_cuda(u)
        if tuple(u.shape) != self.shape or u.dtype != self.dtype:
            raise ValueError(f"expected {self.shape} {self.dtype}, got {tuple(u.shape)} {u.dtype}")
        lib = N.lib()
        ws = workspace(lib.mjx_spec3d_ws_bytes(*self.shape, self.code), self.device, "spec3d")
        out = torch.empty_like(u)
        N.check("mjx_spectral_apply3d", lib.mjx_spectral_apply3d(
            N.ptr(self.buf), C.byref(self.cgrid), self.code, float(D), float(h), int(mult), int(n_steps),
            N.ptr(u), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(self.device)))
        return out


_plans3d: Dict[tuple, SpectralPlan3D] = {}


def get_plan3d(nz, ny, nx, dz, dy, dx, symbol="spectral", dtype=torch.float64, device=None) -> SpectralPlan3D:
    dev = _device(device)
    key = (int(nz), int(ny), int(nx), float(dz), float(dy), float(dx), symbol, dtype, str(dev))
    p = _plans3d.get(key)
    if p is None:
        p = SpectralPlan3D(nz, ny, nx, dz, dy, dx, symbol, dtype, dev)
        _plans3d[key] = p
    return p


def fft_cn_step_3d(u0: torch.Tensor, D: float, dx: float, dt: float, n_steps: int = 1,
                   symbol: str = "spectral", dy: Optional[float] = None,
                   dz: Optional[float] = None) -> torch.Tensor:
    """3D Crank-Nicolson diffusion steps u <- real(ifftn(G fftn(u))),
    G = (1 + dt D lam/2)/(1 - dt D lam/2), lam = -(kx^2 + ky^2 + kz^2) by default
    (benchmarks/sisc/bench_3d_feasibility.py:71-87); each step a full transform pair."""
    nz, ny, nx = u0.shape
    plan = get_plan3d(nz, ny, nx, dz or dx, dy or dx, dx, symbol, u0.dtype, u0.device)
    return plan.apply(u0, D, dt, N.MULT_CN, n_steps)


def solve_helmholtz_3d(rhs: torch.Tensor, D: float, dt: float, dx: float, symbol: str = "fd",
                       dy: Optional[float] = None, dz: Optional[float] = None) -> torch.Tensor:
    """(I - dt D Lap) u = rhs on a periodic box (|denominator| clamped at 1e-14)."""
    nz, ny, nx = rhs.shape
    plan = get_plan3d(nz, ny, nx, dz or dx, dy or dx, dx, symbol, rhs.dtype, rhs.device)
    return plan.apply(rhs, D, dt, N.MULT_HELMHOLTZ)
