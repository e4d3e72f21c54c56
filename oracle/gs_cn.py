"""Oracle: the Gray-Scott benchmark's fixed-step methods.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  NumPy FP64 restatements
of benchmarks/benchmark_gray_scott.py:
* 162-228 (cn_newton_step_jit): per step the CN residual with pseudo-spectral (or
  any given) Laplacian eigenvalues, the exact periodic inverse of
  (I - dt/2 D Lap) as the preconditioner, u <- u + M^-1(-res), while
  max|res_u| + max|res_v| > tol and i < max_iter, starting from u_old with
  res_norm = 1;
* 268-296 (imex_step / imex_solve): explicit Euler half step of the reaction,
  exact exponential diffusion by FFT, explicit Euler half step;
* 93-131 (rk4_rhs / rk4_step / rk4_solve): classical RK4 with the Laplacian by FFT.
"""

from __future__ import annotations

import numpy as np


def spectral_symbol(n, dx):
    """benchmarks/benchmark_gray_scott.py:53-56: -(kx^2 + ky^2), k = 2 pi fftfreq(n, dx)."""
    k = np.fft.fftfreq(n, dx) * 2 * np.pi
    KX, KY = np.meshgrid(k, k, indexing="ij")
    return -(KX ** 2 + KY ** 2)


def benchmark_ic(n):
    """benchmarks/benchmark_gray_scott.py:59-68 (numpy's legacy seed 42 stream): noise about
    (1, 0.25) and a 2r x 2r square (r = 10) of (0.5, 0.25) at the centre."""
    rs = np.random.RandomState(42)
    u0 = np.ones((n, n)) - 0.5 * rs.rand(n, n) * 0.1
    v0 = 0.25 * np.ones((n, n)) + 0.5 * rs.rand(n, n) * 0.1
    c, r = n // 2, 10
    u0[c - r:c + r, c - r:c + r] = 0.5
    v0[c - r:c + r, c - r:c + r] = 0.25
    return u0, v0


def cn_newton_step(u_old, v_old, lam, Du, Dv, F, k, dt, tol=1e-8, max_iter=10):
    """One step; returns (u, v, iterations)."""
    fft2, ifft2 = np.fft.fft2, np.fft.ifft2
    pu = 1.0 / (1.0 - 0.5 * dt * Du * lam)
    pv = 1.0 / (1.0 - 0.5 * dt * Dv * lam)
    lap_uo = np.real(ifft2(lam * fft2(u_old)))
    lap_vo = np.real(ifft2(lam * fft2(v_old)))
    uvv_o = u_old * v_old * v_old
    Ruo, Rvo = -uvv_o + F * (1 - u_old), uvv_o - (F + k) * v_old
    u, v = u_old.copy(), v_old.copy()
    res_norm, i = 1.0, 0
    while res_norm > tol and i < max_iter:
        lap_u = np.real(ifft2(lam * fft2(u)))
        lap_v = np.real(ifft2(lam * fft2(v)))
        uvv = u * v * v
        res_u = u - u_old - 0.5 * dt * (Du * (lap_u + lap_uo) + (-uvv + F * (1 - u)) + Ruo)
        res_v = v - v_old - 0.5 * dt * (Dv * (lap_v + lap_vo) + (uvv - (F + k) * v) + Rvo)
        u = u + np.real(ifft2(pu * fft2(-res_u)))
        v = v + np.real(ifft2(pv * fft2(-res_v)))
        res_norm = np.max(np.abs(res_u)) + np.max(np.abs(res_v))
        i += 1
    return u, v, i


def cn_solve(u0, v0, lam, Du, Dv, F, k, dt, n_steps, tol=1e-8, max_iter=10):
    """n_steps steps (cn_solve_jit, 216-221); returns (u, v, per-step iteration counts)."""
    u, v, its = u0, v0, []
    for _ in range(n_steps):
        u, v, it = cn_newton_step(u, v, lam, Du, Dv, F, k, dt, tol, max_iter)
        its.append(it)
    return u, v, its


def strang_exp_step(u, v, lam, Du, Dv, F, k, dt):
    """benchmarks/benchmark_gray_scott.py:268-289."""
    uvv = u * v * v
    u = u + 0.5 * dt * (-uvv + F * (1 - u))
    v = v + 0.5 * dt * (uvv - (F + k) * v)
    u = np.real(np.fft.ifft2(np.fft.fft2(u) * np.exp(dt * Du * lam)))
    v = np.real(np.fft.ifft2(np.fft.fft2(v) * np.exp(dt * Dv * lam)))
    uvv = u * v * v
    u = u + 0.5 * dt * (-uvv + F * (1 - u))
    v = v + 0.5 * dt * (uvv - (F + k) * v)
    return u, v


def strang_exp_solve(u0, v0, lam, Du, Dv, F, k, dt, n_steps):
    """imex_solve (291-296): n_steps steps."""
    u, v = u0, v0
    for _ in range(n_steps):
        u, v = strang_exp_step(u, v, lam, Du, Dv, F, k, dt)
    return u, v


def rk4_rhs(u, v, lam, Du, Dv, F, k):
    """benchmarks/benchmark_gray_scott.py:93-106."""
    lap_u = np.real(np.fft.ifft2(lam * np.fft.fft2(u)))
    lap_v = np.real(np.fft.ifft2(lam * np.fft.fft2(v)))
    uvv = u * v * v
    return Du * lap_u - uvv + F * (1 - u), Dv * lap_v + uvv - (F + k) * v


def rk4_solve(u0, v0, lam, Du, Dv, F, k, dt, n_steps):
    """rk4_step / rk4_solve (108-125)."""
    u, v = u0, v0
    f = lambda a, b: rk4_rhs(a, b, lam, Du, Dv, F, k)  # noqa: E731
    for _ in range(n_steps):
        k1u, k1v = f(u, v)
        k2u, k2v = f(u + 0.5 * dt * k1u, v + 0.5 * dt * k1v)
        k3u, k3v = f(u + 0.5 * dt * k2u, v + 0.5 * dt * k2v)
        k4u, k4v = f(u + dt * k3u, v + dt * k3v)
        u = u + dt / 6 * (k1u + 2 * k2u + 2 * k3u + k4u)
        v = v + dt / 6 * (k1v + 2 * k2v + 2 * k3v + k4v)
    return u, v


def rk4_dt(n, Du, Dv, dx):
    """0.9 of the RK4 stability limit 2.8 / (max(Du, Dv) max|lam|) (79-90)."""
    lam = spectral_symbol(n, dx)
    return 0.9 * 2.8 / (max(Du, Dv) * float(np.max(-lam)))
