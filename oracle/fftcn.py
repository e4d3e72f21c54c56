"""Oracle: FFT Crank-Nicolson on a periodic box.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restates the FFT-CN
step the reference benchmarks use (it is not a function of the moljax
package itself):

* ``benchmarks/benchmark_vs_scipy.py:74-114`` -- 2D, pseudo-spectral symbol
  -(kx^2+ky^2), ``cn_factor = (1 + dt D lam/2) / (1 - dt D lam/2)``, each step
  ``real(ifft2(fft2(u) * cn_factor))``;
* ``benchmarks/sisc/bench_precision_fp32_fp64.py:41-100`` -- the same at
  128^2, D=0.1, T=0.1 for a range of dt (the published error table);
* ``benchmarks/benchmark_solver_comparison.py:152-163`` -- the 1D form with advection,
  and its exponential Strang splitting (190-215) and SciPy Radau comparison (67-121);
* ``benchmarks/sisc/bench_3d_feasibility.py:56-87`` -- 3D, N^3 points of
  x = j L/N, D = 0.1, 10 steps to T = 0.01, max error vs the analytic decay
  exp(-12 pi^2 D T) sin sin sin.
"""

from __future__ import annotations

import numpy as np

from oracle.mol import fd_symbol_1d, spectral_symbol_1d


def node_grid_ic(n, L=1.0):
    """u0 = sin(2 pi x) sin(2 pi y) on x = j L/n, meshgrid 'ij' (benchmark_vs_scipy.py:62-65)."""
    x = np.linspace(0.0, L, n, endpoint=False)
    X, Y = np.meshgrid(x, x, indexing="ij")
    return np.sin(2 * np.pi * X) * np.sin(2 * np.pi * Y)


def symbol_2d(n0, n1, d0, d1, kind="spectral"):
    """Laplacian eigenvalues on an (n0, n1) periodic grid, fftfreq order."""
    f = spectral_symbol_1d if kind == "spectral" else fd_symbol_1d
    return f(n0, d0)[:, None] + f(n1, d1)[None, :]


def cn_factor(lam, D, dt):
    """benchmarks/benchmark_vs_scipy.py:74-81."""
    return (1.0 + 0.5 * dt * D * lam) / (1.0 - 0.5 * dt * D * lam)


def fft_cn_2d(u0, D, dx, dt, n_steps, kind="spectral", dy=None):
    """benchmarks/benchmark_vs_scipy.py:83-91 / 99-114: n_steps one-by-one CN steps."""
    dy = dx if dy is None else dy
    lam = symbol_2d(u0.shape[0], u0.shape[1], dy, dx, kind)
    G = cn_factor(lam, D, dt)
    u = np.array(u0, dtype=np.float64, copy=True)
    for _ in range(n_steps):
        u = np.real(np.fft.ifft2(np.fft.fft2(u) * G))
    return u


def fft_cn_1d(u0, D, dx, dt, n_steps, kind="spectral", v=0.0):
    """benchmarks/benchmark_solver_comparison.py:145-163 (v != 0 adds -i k v)."""
    n = u0.shape[0]
    k = 2 * np.pi * np.fft.fftfreq(n, dx)
    lam = -(k * k) if kind == "spectral" else fd_symbol_1d(n, dx)
    L = D * lam + v * (-1j * k)
    G = (1 + 0.5 * dt * L) / (1 - 0.5 * dt * L)
    u = np.array(u0, dtype=np.float64, copy=True)
    for _ in range(n_steps):
        u = np.real(np.fft.ifft(np.fft.fft(u) * G))
    return u


def solver_comparison_ic(n=1024):
    """u0 = exp(-100 (x - 0.5)^2) on x = j/n (benchmarks/benchmark_solver_comparison.py:55-58)."""
    x = np.linspace(0, 1, n, endpoint=False)
    return np.exp(-100 * (x - 0.5) ** 2)


def strang_exp_1d(u0, D, v, dx, dt, n_steps):
    """benchmarks/benchmark_solver_comparison.py:190-215 (imex_step / imex_solve): per step
    exp(dt/2 v (-i k)), exp(dt D (-k^2)), exp(dt/2 v (-i k)), each a transform pair keeping
    the real part."""
    n = u0.shape[0]
    k = 2 * np.pi * np.fft.fftfreq(n, dx)
    ea = np.exp(0.5 * dt * v * (-1j * k))
    ed = np.exp(dt * D * (-(k * k)))
    u = np.array(u0, dtype=np.float64, copy=True)
    for _ in range(n_steps):
        u = np.real(np.fft.ifft(np.fft.fft(u) * ea))
        u = np.real(np.fft.ifft(np.fft.fft(u) * ed))
        u = np.real(np.fft.ifft(np.fft.fft(u) * ea))
    return u


def radau_advdiff_1d(u0, D, v, t_final, rtol=1e-6, atol=1e-8):
    """The comparison solution of benchmarks/benchmark_solver_comparison.py:67-121: SciPy
    Radau on the periodic FD semi-discretisation D D2 u - v D1 u (central D1), dense
    matrices; returns (final state, number of output times)."""
    from scipy.integrate import solve_ivp
    n = u0.shape[0]
    dx = 1.0 / n
    D2 = np.zeros((n, n))
    D1 = np.zeros((n, n))
    for i in range(n):
        D2[i, (i - 1) % n], D2[i, i], D2[i, (i + 1) % n] = 1.0, -2.0, 1.0
        D1[i, (i - 1) % n], D1[i, (i + 1) % n] = -1.0, 1.0
    D2 /= dx ** 2
    D1 /= 2 * dx
    sol = solve_ivp(lambda t, u: D * D2 @ u - v * D1 @ u, [0, t_final], u0, method="Radau", rtol=rtol, atol=atol)
    return sol.y[:, -1], len(sol.t)


def analytic_decay(u0, D, T):
    """exp(-8 pi^2 D T) u0 (benchmark_vs_scipy.py:67-68)."""
    return np.exp(-8 * np.pi ** 2 * D * T) * u0


def node_grid_ic_3d(n, L=1.0):
    """u0 = sin(2 pi x) sin(2 pi y) sin(2 pi z), meshgrid 'ij' (bench_3d_feasibility.py:59-63)."""
    x = np.linspace(0.0, L, n, endpoint=False)
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    return np.sin(2 * np.pi * X) * np.sin(2 * np.pi * Y) * np.sin(2 * np.pi * Z)


def fft_cn_3d(u0, D, dx, dt, n_steps):
    """bench_3d_feasibility.py:70-87: lam = -(KX^2+KY^2+KZ^2), each step
    real(ifftn(G fftn(u)))."""
    n0, n1, n2 = u0.shape
    k0 = np.fft.fftfreq(n0, dx) * 2 * np.pi
    k1 = np.fft.fftfreq(n1, dx) * 2 * np.pi
    k2 = np.fft.fftfreq(n2, dx) * 2 * np.pi
    lam = -(k0[:, None, None] ** 2 + k1[None, :, None] ** 2 + k2[None, None, :] ** 2)
    G = cn_factor(lam, D, dt)
    u = np.array(u0, dtype=np.float64, copy=True)
    for _ in range(n_steps):
        u = np.real(np.fft.ifftn(G * np.fft.fftn(u)))
    return u
