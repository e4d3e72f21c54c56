"""Dirichlet spectral solvers (moljax/core/fft_nonperiodic.py drop-in, DST-I part).

``dst_I_fast`` / ``idst_I_fast`` transform along the last axis of a CUDA
tensor of any leading shape; the solvers (Poisson, Helmholtz, ETD1) run the
forward transform, the pointwise multiplier and the inverse transform in one
native kernel launch (``mjx_dst1``).  Lengths N with 2(N+1) a power of two use
the Stockham FFT directly; other N use Bluestein's chirp-z form on the same
FFT (N <= 1023; N = 2^k - 1 up to 2047).  The Neumann solvers run the same way on
the orthonormal DCT-II (``mjx_dct2``: N <= 1024, or N a power of two <= 2048).
The mixed Dirichlet-Neumann case has its symbol (``laplacian_symbol_mixed_dn``)
but no transform, as in the reference.
"""

from __future__ import annotations

import ctypes as C
import math
from typing import Dict, NamedTuple

import torch

from moljax_gb300 import _native as N

_plans: Dict[tuple, torch.Tensor] = {}
PLAIN, HELMHOLTZ, POISSON, ETD1 = 0, 1, 2, 3


class BCType:
    DIRICHLET = "dirichlet"
    NEUMANN = "neumann"
    MIXED_DN = "mixed_dn"
    MIXED_ND = "mixed_nd"


class NonperiodicFFTCache(NamedTuple):
    """fft_nonperiodic.py NonperiodicFFTCache: N, dx, bc type, eigenvalues, k."""
    N: int
    dx: float
    bc_type: str
    laplacian_symbol: torch.Tensor
    k: torch.Tensor


def _plan(n: int, dtype, device, kind: str = "dst1") -> torch.Tensor:
    key = (kind, int(n), dtype, str(device))
    p = _plans.get(key)
    if p is None:
        lib = N.lib()
        code = N.dtype_code(dtype)
        nb = getattr(lib, f"mjx_{kind}_plan_bytes")(int(n), code)
        if nb == 0:
            raise ValueError(f"{kind} length {n} not supported" + (
                " (1 <= N <= 1023, or N = 2^k - 1 <= 2047)" if kind == "dst1"
                else " (1 <= N <= 1024, or N a power of two <= 2048)"))
        p = torch.empty(nb, dtype=torch.uint8, device=device)
        with torch.cuda.device(device):
            N.check(f"mjx_{kind}_plan_init", getattr(lib, f"mjx_{kind}_plan_init")(
                N.ptr(p), int(n), code, N.stream_ptr(device)))
        _plans[key] = p
    return p


def _run(x: torch.Tensor, mode: int, lam=None, h: float = 0.0, D: float = 0.0,
         scale: float = 1.0, second=None, kind: str = "dst1") -> torch.Tensor:
    N.require_cuda(x)
    if x.dtype not in (torch.float32, torch.float64):
        raise TypeError("DST-I needs float32 or float64 data")
    n = x.shape[-1]
    rows = x.reshape(-1, n).contiguous()
    nrows = rows.shape[0]
    if second is not None:  # ETD1: rows of u then rows of N(u)
        rows = torch.cat([rows, second.reshape(-1, n).to(x.dtype)]).contiguous()
    out = torch.empty((nrows, n), dtype=x.dtype, device=x.device)
    lam_t = None
    if lam is not None:
        lam_t = torch.as_tensor(lam, dtype=x.dtype).to(x.device).reshape(-1).contiguous()
        if lam_t.numel() != n:
            raise ValueError("symbol length must equal the transform length")
    plan = _plan(n, x.dtype, x.device, kind)
    N.check(f"mjx_{kind}", getattr(N.lib(), f"mjx_{kind}")(
        N.ptr(plan), int(n), int(nrows), N.dtype_code(x.dtype), int(mode), N.ptr(rows),
        N.ptr(out), N.ptr(lam_t), float(h), float(D), float(scale), N.stream_ptr(x.device)))
    return out.reshape(x.shape)


def dst_I_fast(x: torch.Tensor) -> torch.Tensor:
    """X[k] = sum_n x[n] sin(pi (k+1)(n+1)/(N+1)) along the last axis (fft_nonperiodic.py:97-122)."""
    return _run(x, PLAIN)


def idst_I_fast(X: torch.Tensor) -> torch.Tensor:
    """Inverse DST-I = 2/(N+1) DST-I (fft_nonperiodic.py:125-133)."""
    return _run(X, PLAIN, scale=2.0 / (X.shape[-1] + 1))


def laplacian_symbol_dirichlet(N_: int, dx: float, dtype=torch.float64, device=None) -> torch.Tensor:
    """lambda_k = -4/dx^2 sin^2(pi k / (2(N+1))), k = 1..N (fft_nonperiodic.py:140-162)."""
    k = torch.arange(1, N_ + 1, dtype=torch.float64)
    lam = -4.0 / (dx * dx) * torch.sin(math.pi * k / (2 * (N_ + 1))) ** 2
    return lam.to(dtype=dtype, device=device if device is not None else "cpu")


def laplacian_symbol_neumann(N_: int, dx: float, dtype=torch.float64, device=None) -> torch.Tensor:
    """lambda_k = -4/dx^2 sin^2(pi k / (2N)), k = 0..N-1; lambda_0 = 0 (fft_nonperiodic.py:165-183)."""
    k = torch.arange(N_, dtype=torch.float64)
    lam = -4.0 / (dx * dx) * torch.sin(math.pi * k / (2 * N_)) ** 2
    return lam.to(dtype=dtype, device=device if device is not None else "cpu")


def laplacian_symbol_mixed_dn(N_: int, dx: float, dtype=torch.float64, device=None) -> torch.Tensor:
    """lambda_k = -4/dx^2 sin^2(pi (2k-1) / (4N)), k = 1..N (fft_nonperiodic.py:186-196)."""
    k = torch.arange(1, N_ + 1, dtype=torch.float64)
    lam = -4.0 / (dx * dx) * torch.sin(math.pi * (2 * k - 1) / (4 * N_)) ** 2
    return lam.to(dtype=dtype, device=device if device is not None else "cpu")


def create_nonperiodic_fft_cache(N_: int, dx: float, bc_type=BCType.DIRICHLET,
                                 dtype=torch.float64, device=None) -> NonperiodicFFTCache:
    """fft_nonperiodic.py:200-241."""
    bc = str(getattr(bc_type, "value", bc_type)).lower()
    if bc == BCType.DIRICHLET:
        lam = laplacian_symbol_dirichlet(N_, dx, dtype, device)
        k = torch.arange(1, N_ + 1, dtype=dtype)
    elif bc == BCType.NEUMANN:
        lam = laplacian_symbol_neumann(N_, dx, dtype, device)
        k = torch.arange(N_, dtype=dtype)
    elif bc == BCType.MIXED_DN:
        lam = laplacian_symbol_mixed_dn(N_, dx, dtype, device)
        k = torch.arange(1, N_ + 1, dtype=dtype)
    else:
        raise ValueError(f"Unsupported BC type: {bc_type}")
    return NonperiodicFFTCache(N_, dx, bc, lam, k.to(lam.device))


def solve_poisson_dirichlet(rhs: torch.Tensor, laplacian_symbol) -> torch.Tensor:
    """Lap u = f with u = 0 at both ends (fft_nonperiodic.py:244-271)."""
    return _run(rhs, POISSON, laplacian_symbol)


def solve_helmholtz_dirichlet(rhs: torch.Tensor, laplacian_symbol, dt: float, D: float) -> torch.Tensor:
    """(I - dt D Lap) u = f with Dirichlet ends (fft_nonperiodic.py:308-330)."""
    return _run(rhs, HELMHOLTZ, laplacian_symbol, h=dt, D=D)


def etd1_dirichlet(u: torch.Tensor, N_u: torch.Tensor, eigenvalues, dt: float) -> torch.Tensor:
    """exp(z) u^ + dt phi1(z) N^ with z = dt * eigenvalues (fft_nonperiodic.py:360-398)."""
    return _run(u, ETD1, eigenvalues, h=dt, second=N_u)


def dst_I(x: torch.Tensor) -> torch.Tensor:
    """2 * sum_n x[n] sin(pi (k+1)(n+1)/(N+1)) (fft_nonperiodic.py:49-77: twice dst_I_fast)."""
    return _run(x, PLAIN, scale=2.0)


def idst_I(X: torch.Tensor) -> torch.Tensor:
    """dst_I(X) / (N+1) (fft_nonperiodic.py:80-94)."""
    return _run(X, PLAIN, scale=2.0 / (X.shape[-1] + 1))


# ---------------------------------------------------------------- Neumann (DCT-II)
DCT_FWD, DCT_INV, DCT_HELMHOLTZ, DCT_POISSON, DCT_ETD1 = 0, 1, 2, 3, 4


def dct(x: torch.Tensor, type: int = 2, norm: str = "ortho") -> torch.Tensor:  # noqa: A002
    """Orthonormal DCT-II along the last axis (jax.scipy.fft.dct(x, type=2, norm='ortho'))."""
    if type != 2 or norm != "ortho":
        raise NotImplementedError("only the orthonormal DCT-II is built")
    return _run(x, DCT_FWD, kind="dct2")


def idct(X: torch.Tensor, type: int = 2, norm: str = "ortho") -> torch.Tensor:  # noqa: A002
    """Inverse of the orthonormal DCT-II (DCT-III) along the last axis."""
    if type != 2 or norm != "ortho":
        raise NotImplementedError("only the orthonormal DCT-II is built")
    return _run(X, DCT_INV, kind="dct2")


def solve_poisson_neumann(rhs: torch.Tensor, laplacian_symbol) -> torch.Tensor:
    """Lap u = f with zero-flux ends; the null mode is set to zero (fft_nonperiodic.py:274-305)."""
    return _run(rhs, DCT_POISSON, laplacian_symbol, kind="dct2")


def solve_helmholtz_neumann(rhs: torch.Tensor, laplacian_symbol, dt: float, D: float) -> torch.Tensor:
    """(I - dt D Lap) u = f with zero-flux ends (fft_nonperiodic.py:333-355)."""
    return _run(rhs, DCT_HELMHOLTZ, laplacian_symbol, h=dt, D=D, kind="dct2")


def etd1_neumann(u: torch.Tensor, N_u: torch.Tensor, eigenvalues, dt: float) -> torch.Tensor:
    """exp(z) u^ + dt phi1(z) N^ in the DCT basis (fft_nonperiodic.py:401-437)."""
    return _run(u, DCT_ETD1, eigenvalues, h=dt, second=N_u, kind="dct2")


def check_compatibility_neumann(rhs: torch.Tensor, tol: float = 1e-10) -> bool:
    """|sum(f)| < tol (fft_nonperiodic.py:444-452)."""
    return abs(float(rhs.sum())) < tol


def project_to_compatible(rhs: torch.Tensor) -> torch.Tensor:
    """f - mean(f) (fft_nonperiodic.py:455-461)."""
    return rhs - rhs.mean()
