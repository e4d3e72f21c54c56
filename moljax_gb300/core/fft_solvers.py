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


def _pow2(n: int) -> bool:
    return n >= 1 and (n & (n - 1)) == 0


class GeneralSpectralPlan:
    """Periodic (ny, nx) grid of any supported size (powers of two up to 4096, other sizes up
    to 2048): the full-spectrum path of ``mjx_spectral_apply_general2d`` (row DFTs by
    Stockham or Bluestein, transposes, column DFTs and the multiplier).  Same ``apply`` as
    ``SpectralPlan``; the fused device loops (IMEX, ETD) take powers of two, their
    host-driven forms run on this plan."""

    general = True

    def __init__(self, ny: int, nx: int, dy: float, dx: float, symbol: str = "fd",
                 dtype: torch.dtype = torch.float64, device=None):
        N.require_cuda()
        self.ny, self.nx, self.dy, self.dx = int(ny), int(nx), float(dy), float(dx)
        self.symbol, self.dtype, self.device = symbol, dtype, _device(device)
        self.code = N.dtype_code(dtype)
        lib = N.lib()
        self.cgrid = N.Grid2DC(self.ny, self.nx, self.dy, self.dx)
        bufs = []
        for n in (self.ny, self.nx):
            nb = lib.mjx_dftn_plan_bytes(n, self.code)
            if nb == 0:
                raise ValueError(f"unsupported grid {ny}x{nx}: lengths must be powers of two <= 4096 or <= 2048")
            b = torch.empty(nb, dtype=torch.uint8, device=self.device)
            with torch.cuda.device(self.device):
                N.check("mjx_dftn_plan_init", lib.mjx_dftn_plan_init(N.ptr(b), n, self.code,
                                                                     N.stream_ptr(self.device)))
            bufs.append(b)
        self.buf_y, self.buf_x = bufs
        self.buf = self.buf_y  # the power-of-two entry points reject this grid by its shape
        from moljax_gb300.core import autotune
        autotune.tune_lengths([(self.nx, self.ny, self.buf_x), (self.ny, self.nx, self.buf_y)], dtype, self.device)

    def ws_bytes(self, nfields: int) -> int:
        return N.lib().mjx_spectral_general2d_ws_bytes(self.ny, self.nx, nfields, self.code)

    def apply(self, x: torch.Tensor, D, h: float, mult: int, out: Optional[torch.Tensor] = None,
              vx=None, vy=None, table: Optional[torch.Tensor] = None):
        """out_f = real(IFFT2(m(h, D_f, ...) FFT2(x_f))) for x of shape (ny, nx) or (nf, ny, nx)."""
        x3 = x.reshape(-1, self.ny, self.nx).contiguous()
        N.require_cuda(x3)
        if x3.dtype != self.dtype:
            raise TypeError(f"plan dtype {self.dtype} does not match {x3.dtype}")
        nf = x3.shape[0]

        def per_field(v):
            if v is None:
                return [0.0] * nf
            return [float(v)] * nf if not isinstance(v, (list, tuple)) else [float(t) for t in v]
        Ds, vxs, vys = per_field(D), per_field(vx), per_field(vy)
        out3 = torch.empty_like(x3) if out is None else out.reshape(-1, self.ny, self.nx)
        sym = SYMBOLS[self.symbol]
        for i in range(0, nf, 4):
            j = min(nf, i + 4)
            ws = workspace(self.ws_bytes(j - i), self.device, "general")
            arr = lambda v: (C.c_double * (j - i))(*v[i:j])  # noqa: E731
            N.check("mjx_spectral_apply_general2d", N.lib().mjx_spectral_apply_general2d(
                N.ptr(self.buf_y), N.ptr(self.buf_x), C.byref(self.cgrid), sym, self.code, j - i,
                arr(Ds), arr(vxs), arr(vys), float(h), int(mult),
                N.ptr(table) if table is not None else None, N.ptr(x3[i:j]), N.ptr(out3[i:j]),
                N.ptr(ws), ws.numel(), N.stream_ptr(self.device)))
        return out3.reshape(x.shape)


def get_plan(ny, nx, dy, dx, symbol="fd", dtype=torch.float64, device=None):
    """The spectral plan of a periodic (ny, nx) grid: the fused power-of-two passes, or the
    general full-spectrum path for other sizes."""
    dev = _device(device)
    key = (int(ny), int(nx), float(dy), float(dx), symbol, dtype, str(dev))
    p = _plans.get(key)
    if p is None:
        if _pow2(int(ny)) and _pow2(int(nx)) and ny >= 2 and nx >= 2:
            p = SpectralPlan(ny, nx, dy, dx, symbol, dtype, dev)
        else:
            p = GeneralSpectralPlan(ny, nx, dy, dx, symbol, dtype, dev)
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


def build_wavenumbers_2d(ny: int, nx: int, dy: float, dx: float, dtype=torch.float64):
    """moljax/core/fft_solvers.py:67-94: (kx, ky), each (ny, nx), 2 pi fftfreq."""
    kx = build_wavenumbers_1d(nx, dx, dtype)[None, :].expand(ny, nx).contiguous()
    ky = build_wavenumbers_1d(ny, dy, dtype)[:, None].expand(ny, nx).contiguous()
    return kx, ky


class FFTCache1D(NamedTuple):
    """moljax/core/fft_solvers.py:31-35 plus the native plan (a 2-row grid whose rows
    carry the same field, so that its y modes are zero)."""
    laplacian_symbol: torch.Tensor
    k: torch.Tensor
    plan: SpectralPlan


def _plan_1d(nx: int, dx: float, dtype, device=None) -> SpectralPlan:
    return get_plan(2, nx, dx, dx, "fd", dtype, device)


def create_fft_cache_1d(grid: Grid1D, dtype=torch.float64, device=None) -> FFTCache1D:
    """moljax/core/fft_solvers.py:161-178."""
    dev = _device(device)
    lam = laplacian_symbol_1d(grid.nx, grid.dx, dtype).to(dev)
    plan = _plan_1d(grid.nx, grid.dx, dtype, dev)
    lam._mjx_plan = plan
    return FFTCache1D(lam, build_wavenumbers_1d(grid.nx, grid.dx, dtype).to(dev), plan)


def create_fft_cache(grid, dtype=torch.float64, device=None):
    """moljax/core/fft_solvers.py:201-215."""
    if isinstance(grid, Grid1D):
        return create_fft_cache_1d(grid, dtype, device)
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


def _apply_1d(plan: SpectralPlan, u: torch.Tensor, D, h: float, mult: int) -> torch.Tensor:
    """A multiplier on 1D fields (..., nx) through the 2-row plan (both rows the same field)."""
    u2 = u.reshape(-1, 1, u.shape[-1]).expand(-1, 2, -1).contiguous()
    return plan.apply(u2, D, h, mult)[:, 0].reshape(u.shape).clone()


def solve_helmholtz_1d(rhs_interior: torch.Tensor, laplacian_symbol, dt: float, D: float):
    """(I - dt D Lap) u = rhs on a periodic 1D interior (moljax/core/fft_solvers.py:222-258)."""
    nx = rhs_interior.shape[-1]
    plan = getattr(laplacian_symbol, "plan", None) or getattr(laplacian_symbol, "_mjx_plan", None)
    if plan is None:
        raise NotImplementedError("solve_helmholtz_1d needs a symbol made by create_fft_cache_1d")
    if plan.nx != nx or plan.ny != 2:
        raise ValueError("symbol/grid shape mismatch")
    if plan.dtype != rhs_interior.dtype:
        plan = get_plan(2, nx, plan.dy, plan.dx, plan.symbol, rhs_interior.dtype, plan.device)
    return _apply_1d(plan, rhs_interior, D, dt, N.MULT_HELMHOLTZ)


def solve_helmholtz_2d(rhs_interior: torch.Tensor, laplacian_symbol, dt: float, D: float):
    """(I - dt D Lap) u = rhs on the interior (moljax/core/fft_solvers.py:261-294)."""
    ny, nx = rhs_interior.shape[-2:]
    plan = _plan_of(laplacian_symbol, ny, nx, rhs_interior.dtype)
    return plan.apply(rhs_interior.contiguous(), D, dt, N.MULT_HELMHOLTZ)


def solve_helmholtz(rhs_interior, laplacian_symbol, dt, D):
    """moljax/core/fft_solvers.py:297-320."""
    if rhs_interior.ndim == 1:
        return solve_helmholtz_1d(rhs_interior, laplacian_symbol, dt, D)
    return solve_helmholtz_2d(rhs_interior, laplacian_symbol, dt, D)


def extract_interior(f_padded, grid):
    """moljax/core/fft_solvers.py:327-342."""
    return f_padded[grid.interior_slice]


def embed_interior(u_interior, grid, padded_template):
    """moljax/core/fft_solvers.py:345-365 (ghosts from the template)."""
    out = padded_template.clone()
    out[grid.interior_slice] = u_interior
    return out


def solve_diffusion_fft_field(rhs_padded, grid, dt: float, D: float, fft_cache):
    """(I - dt D Lap) u = rhs for one padded field; ghosts from rhs (fft_solvers.py:368-403)."""
    u = solve_helmholtz(extract_interior(rhs_padded, grid).contiguous(), fft_cache.laplacian_symbol, dt, D)
    return embed_interior(u, grid, rhs_padded)


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


def apply_diffusion_fft(state, grid, dt: float, diffusivities, fft_cache):
    """Implicit Euler diffusion step u <- (I - dt D Lap)^-1 u (fft_solvers.py:448-474)."""
    if isinstance(grid, Grid1D):
        return {n: (solve_diffusion_fft_field(f, grid, dt, diffusivities[n], fft_cache)
                    if diffusivities.get(n, 0.0) > 1e-14 else f) for n, f in state.items()}
    return apply_diffusion_inverse_fft(state, grid, dt, diffusivities, fft_cache)


def diffusion_rhs_fft(state, grid, diffusivities, fft_cache):
    """D Lap u of each field through the FFT symbol, ghosts zero (fft_solvers.py:619-660)."""
    out = {}
    for n, f in state.items():
        D = diffusivities.get(n, 0.0)
        if D > 1e-14:
            fi = extract_interior(f, grid).contiguous()
            if fi.ndim == 1:
                lap = _apply_1d(_plan_of(fft_cache, 2, fi.shape[-1], fi.dtype), fi, D, 1.0, N.MULT_LAP)
            else:
                lap = _plan_of(fft_cache, fi.shape[0], fi.shape[1], fi.dtype).apply(fi, D, 1.0, N.MULT_LAP)
            out[n] = embed_interior(lap, grid, torch.zeros_like(f))
        else:
            out[n] = torch.zeros_like(f)
    return out


# ----------------------------------------------------------------- spectral filters
def exponential_filter_1d(nx: int, strength: float = 36.0, order: int = 36, dtype=torch.float64):
    """sigma(k) = exp(-strength (|k|/k_max)^order), |k| = min(k, n - k) (fft_solvers.py:477-503)."""
    k = torch.arange(nx, dtype=torch.float64)
    kn = torch.minimum(k, nx - k) / (nx // 2)
    kn = torch.clamp(kn, max=1.0)
    return torch.exp(-strength * kn ** order).to(dtype)


def exponential_filter_2d(ny: int, nx: int, strength: float = 36.0, order: int = 36, dtype=torch.float64):
    """Outer product of the 1D filters (fft_solvers.py:506-531)."""
    return torch.outer(exponential_filter_1d(ny, strength, order, dtype),
                       exponential_filter_1d(nx, strength, order, dtype))


def _half_table(kernel: torch.Tensor, ny: int, nx: int, dtype, device) -> torch.Tensor:
    """The real multiplier on the half spectrum equivalent to real(ifft2(K fft2(u))):
    (K(k) + K(-k)) / 2 for kx = 0..nx/2, padded to the plan's row length."""
    K = kernel.to(torch.float64).cpu()
    if K.is_complex():
        raise NotImplementedError("complex filter kernels are not supported")
    if K.ndim == 1:
        K = K[None, :].expand(ny, nx)
    iy = (-torch.arange(ny)) % ny
    ix = (-torch.arange(nx)) % nx
    Km = K[iy][:, ix]
    half = 0.5 * (K + Km)[:, : nx // 2 + 1]
    ldc = ((nx // 2 + 1) + 3) & ~3
    tab = torch.zeros(ny, ldc, dtype=torch.float64)
    tab[:, : nx // 2 + 1] = half
    return tab.to(dtype).to(device).contiguous()


def apply_spectral_filter_interior(u_interior: torch.Tensor, filter_kernel) -> torch.Tensor:
    """real(ifft(sigma * fft(u))) on a 1D or 2D interior (fft_solvers.py:534-556)."""
    u = u_interior.contiguous()
    N.require_cuda(u)
    if u.ndim == 1:
        ny, nx = 2, u.shape[0]
        x = torch.stack([u, u])
    else:
        ny, nx = u.shape
        x = u
    kern = filter_kernel if torch.is_tensor(filter_kernel) else torch.as_tensor(filter_kernel)
    plan = get_plan(ny, nx, 1.0 / ny, 1.0 / nx, "fd", u.dtype, u.device)
    if getattr(plan, "general", False):
        K = kern.to(torch.float64)
        if K.ndim == 1:
            K = K[None, :].expand(ny, nx)
        tab = K.to(u.dtype).to(u.device).contiguous()
        out = plan.apply(x, 1.0, 1.0, N.MULT_TABLE, table=tab)
        return out[0].clone() if u.ndim == 1 else out
    tab = _half_table(kern, ny, nx, u.dtype, u.device)
    out = torch.empty_like(x)
    ws = workspace(plan.ws_bytes(1), plan.device)
    N.check("mjx_spectral_filter2d", N.lib().mjx_spectral_filter2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, 1, N.ptr(tab), N.ptr(x), N.ptr(out),
        N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out[0].clone() if u.ndim == 1 else out


def apply_spectral_filter_field(f_padded, grid, filter_kernel):
    """fft_solvers.py:559-581: filter the interior, ghosts kept."""
    return embed_interior(apply_spectral_filter_interior(extract_interior(f_padded, grid), filter_kernel),
                          grid, f_padded)


def apply_spectral_filter_state(state, grid, filter_kernel, filter_fields=None):
    """fft_solvers.py:584-616: fields with filter_fields[name] False (default True) pass through."""
    return {n: (apply_spectral_filter_field(f, grid, filter_kernel)
                if filter_fields is None or filter_fields.get(n, True) else f) for n, f in state.items()}


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
    if getattr(plan, "general", False):
        for _ in range(int(n_steps)):  # each step a full transform pair
            u = plan.apply(u, D, dt, N.MULT_CN)
        return u
    out = torch.empty_like(u)
    ws = workspace(plan.ws_bytes(1), plan.device)
    N.check("mjx_fft_cn2d", N.lib().mjx_fft_cn2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, float(D), float(dt), int(n_steps),
        N.ptr(u), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out


def _advdiff_1d_apply(plan, x, D: float, v: float, h: float, op: int, out: torch.Tensor):
    """One mjx_advdiff_op2d call on the two identical rows of a 1D field (op 0 solve, 1 h L,
    2 exp(h L), 3 one CN step); the general-size path for other lengths."""
    if getattr(plan, "general", False):
        mult = (N.MULT_ADV_SOLVE, N.MULT_ADV_LAP, N.MULT_ADV_EXP, N.MULT_ADV_CN)[op]
        return plan.apply(x, float(D), h, mult, out=out, vx=float(v), vy=0.0)
    ws = workspace(plan.ws_bytes(1), plan.device)
    D_ = (C.c_double * 1)(float(D))
    vx_ = (C.c_double * 1)(float(v))
    vy_ = (C.c_double * 1)(0.0)
    N.check("mjx_advdiff_op2d", N.lib().mjx_advdiff_op2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, 1, D_, vx_, vy_, float(h), int(op),
        N.ptr(x), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out


def fft_cn_advdiff_1d(u0: torch.Tensor, D: float, v: float, dx: float, dt: float, n_steps: int = 1,
                      symbol: str = "spectral") -> torch.Tensor:
    """Crank-Nicolson steps of the periodic 1D advection-diffusion u_t = D u_xx - v u_x,
    u <- real(ifft(G fft(u))), G = (1 + dt L/2)/(1 - dt L/2), L = D lam - i v k
    (benchmarks/benchmark_solver_comparison.py:145-176, fft_cn_step / fft_cn_solve;
    pseudo-spectral lam = -k^2 by default, as the benchmark).  One native transform pair per
    step (``mjx_advdiff_op2d`` op 3)."""
    u = u0.contiguous()
    N.require_cuda(u)
    if u.ndim != 1:
        raise ValueError("fft_cn_advdiff_1d: a field of shape (nx,)")
    plan = get_plan(2, u.shape[0], dx, dx, symbol, u.dtype, u.device)
    a, b = torch.stack([u, u]), torch.empty(2, u.shape[0], dtype=u.dtype, device=u.device)
    for _ in range(int(n_steps)):
        _advdiff_1d_apply(plan, a, D, v, dt, 3, b)
        a, b = b, a
    return a[0].clone()


def imex_advdiff_1d(u0: torch.Tensor, D: float, v: float, dx: float, dt: float, n_steps: int = 1,
                    symbol: str = "spectral") -> torch.Tensor:
    """Exponential Strang steps of u_t = D u_xx - v u_x: exp(dt/2 (-i v k)), exp(dt D lam),
    exp(dt/2 (-i v k)), each a transform pair keeping the real part
    (benchmarks/benchmark_solver_comparison.py:184-215, imex_step / imex_solve)."""
    u = u0.contiguous()
    N.require_cuda(u)
    if u.ndim != 1:
        raise ValueError("imex_advdiff_1d: a field of shape (nx,)")
    plan = get_plan(2, u.shape[0], dx, dx, symbol, u.dtype, u.device)
    a, b = torch.stack([u, u]), torch.empty(2, u.shape[0], dtype=u.dtype, device=u.device)
    for _ in range(int(n_steps)):
        _advdiff_1d_apply(plan, a, 0.0, v, 0.5 * dt, 2, b)
        _advdiff_1d_apply(plan, b, D, 0.0, dt, 2, a)
        _advdiff_1d_apply(plan, a, 0.0, v, 0.5 * dt, 2, b)
        a, b = b, a
    return a[0].clone()


def gray_scott_strang_exp(u0: torch.Tensor, v0: torch.Tensor, Du: float, Dv: float, F: float, k: float,
                          dt: float, n_steps: int, dx: float, dy: Optional[float] = None,
                          symbol: str = "spectral"):
    """Fixed Strang steps of periodic Gray-Scott as benchmarks/benchmark_gray_scott.py:268-296
    (imex_step / imex_solve): explicit Euler half step of the reaction, exact exponential
    diffusion exp(dt D lam) by FFT, explicit Euler half step; pseudo-spectral Laplacian by
    default, as the benchmark.  One row and one column pass per step (``mjx_gs_strang_exp2d``).
    Returns (u, v)."""
    u0 = u0.contiguous()
    N.require_cuda(u0, v0)
    ny, nx = u0.shape
    dy = dx if dy is None else dy
    plan = get_plan(ny, nx, dy, dx, symbol, u0.dtype, u0.device)
    if getattr(plan, "general", False):
        raise ValueError("gray_scott_strang_exp: grid sides must be powers of two")
    lib = N.lib()
    y = torch.stack([u0, v0.to(u0.dtype)]).contiguous()
    out = torch.empty_like(y)
    ws = workspace(lib.mjx_gs_strang_exp_ws_bytes(ny, nx, plan.code), plan.device, "gs_strang")
    Dc = (C.c_double * 2)(float(Du), float(Dv))
    N.check("mjx_gs_strang_exp2d", lib.mjx_gs_strang_exp2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, Dc, float(F), float(k), float(dt), int(n_steps),
        N.ptr(y), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out[0], out[1]


def gray_scott_rk4_spectral(u0: torch.Tensor, v0: torch.Tensor, Du: float, Dv: float, F: float, k: float,
                            dt: float, n_steps: int, dx: float, dy: Optional[float] = None,
                            symbol: str = "spectral"):
    """Classical RK4 of periodic Gray-Scott with the Laplacian by FFT, as
    benchmarks/benchmark_gray_scott.py:93-131 (rk4_rhs / rk4_step / rk4_solve); pseudo-spectral
    by default.  Per stage one column and one row pass (``mjx_gs_rk4_spectral2d``).
    Returns (u, v)."""
    u0 = u0.contiguous()
    N.require_cuda(u0, v0)
    ny, nx = u0.shape
    dy = dx if dy is None else dy
    plan = get_plan(ny, nx, dy, dx, symbol, u0.dtype, u0.device)
    if getattr(plan, "general", False):
        raise ValueError("gray_scott_rk4_spectral: grid sides must be powers of two")
    lib = N.lib()
    y = torch.stack([u0, v0.to(u0.dtype)]).contiguous()
    out = torch.empty_like(y)
    ws = workspace(lib.mjx_gs_rk4_spectral_ws_bytes(ny, nx, plan.code), plan.device, "gs_rk4")
    Dc = (C.c_double * 2)(float(Du), float(Dv))
    N.check("mjx_gs_rk4_spectral2d", lib.mjx_gs_rk4_spectral2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, Dc, float(F), float(k), float(dt), int(n_steps),
        N.ptr(y), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out[0], out[1]


def gray_scott_cn_newton(u0: torch.Tensor, v0: torch.Tensor, Du: float, Dv: float, F: float, k: float,
                         dt: float, n_steps: int, dx: float, dy: Optional[float] = None, tol: float = 1e-8,
                         max_iter: int = 10, symbol: str = "spectral"):
    """Crank-Nicolson Gray-Scott steps solved by the preconditioned Newton iteration of
    benchmarks/benchmark_gray_scott.py:162-228 (cn_newton_step_jit / cn_solve_jit):
    residual of the CN step, the exact periodic inverse of (I - dt/2 D Lap) as the
    preconditioner, while max|res_u| + max|res_v| > tol and fewer than max_iter
    iterations ran.  The Newton loop of every step runs on the device
    (``mjx_gs_cn_newton2d``); pseudo-spectral Laplacian by default, as the benchmark.
    Returns (u, v, per-step Newton iteration counts)."""
    u0 = u0.contiguous()
    N.require_cuda(u0, v0)
    ny, nx = u0.shape
    dy = dx if dy is None else dy
    plan = get_plan(ny, nx, dy, dx, symbol, u0.dtype, u0.device)
    if getattr(plan, "general", False):
        raise NotImplementedError("gray_scott_cn_newton needs a power-of-two grid")
    y = torch.stack([u0, v0.to(u0.dtype)]).contiguous()
    out = torch.empty_like(y)
    iters = torch.zeros(max(int(n_steps), 1), dtype=torch.int32, device=u0.device)
    lib = N.lib()
    ws = workspace(lib.mjx_gs_cn_ws_bytes(ny, nx, plan.code), plan.device, "gs_cn")
    D = (C.c_double * 2)(float(Du), float(Dv))
    tot, last = C.c_int(0), C.c_double(0.0)
    N.check("mjx_gs_cn_newton2d", lib.mjx_gs_cn_newton2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, D, float(F), float(k), float(dt), int(n_steps),
        float(tol), int(max_iter), N.ptr(y), N.ptr(out), C.cast(C.c_void_p(iters.data_ptr()), C.POINTER(C.c_int)),
        C.byref(tot), C.byref(last), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    return out[0], out[1], iters[:int(n_steps)]


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
        self.cgrid = N.Grid3DC(int(nz), int(ny), int(nx), 0, float(dz), float(dy), float(dx))
        # powers of two >= 2: the fused five-pass form; other lengths: the general path
        self.general = not all(_pow2(n) and n >= 2 for n in self.shape)
        if self.general:
            self.bufs = []
            for n in self.shape:
                nb = lib.mjx_dftn_plan_bytes(n, self.code)
                if nb == 0:
                    raise ValueError(f"unsupported box {nz}x{ny}x{nx}: lengths must be powers of two <= 4096 "
                                     "or <= 2048")
                b = torch.empty(nb, dtype=torch.uint8, device=self.device)
                with torch.cuda.device(self.device):
                    N.check("mjx_dftn_plan_init", lib.mjx_dftn_plan_init(N.ptr(b), n, self.code,
                                                                         N.stream_ptr(self.device)))
                self.bufs.append(b)
            from moljax_gb300.core import autotune
            nz_, ny_, nx_ = self.shape
            autotune.tune_lengths([(nx_, nz_ * ny_, self.bufs[2]), (ny_, nz_ * nx_, self.bufs[1]),
                                   (nz_, ny_ * nx_, self.bufs[0])], dtype, self.device)
            return
        nbytes = lib.mjx_spec3d_plan_bytes(*self.shape, self.code)
        if nbytes == 0:
            raise ValueError(f"unsupported box {nz}x{ny}x{nx}: sizes must be powers of two in [2, 4096]")
        self.buf = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
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
        out = torch.empty_like(u)
        if self.general:
            ws = workspace(lib.mjx_spectral_general3d_ws_bytes(*self.shape, self.code), self.device, "general3d")
            N.check("mjx_spectral_apply_general3d", lib.mjx_spectral_apply_general3d(
                N.ptr(self.bufs[0]), N.ptr(self.bufs[1]), N.ptr(self.bufs[2]), C.byref(self.cgrid),
                SYMBOLS[self.symbol], self.code, float(D), float(h), int(mult), int(n_steps), N.ptr(u),
                N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(self.device)))
            return out
        ws = workspace(lib.mjx_spec3d_ws_bytes(*self.shape, self.code), self.device, "spec3d")
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
