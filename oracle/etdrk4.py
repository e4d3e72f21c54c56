"""Oracle: ETDRK4 (Cox-Matthews) for coupled Gray-Scott on a periodic box.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restates
benchmarks/benchmark_gray_scott.py:336-417: coefficients from the M=32 point
contour mean (compute_etdrk4_coeffs, 336-356) and the coupled step
(etdrk4_step, 369-417), and the phi-function scalar forms of
moljax/core/fft_integrators.py:39-116 used as an independent check.
"""

from __future__ import annotations

import numpy as np

_fft2, _ifft2 = np.fft.fft2, np.fft.ifft2


def set_fft_workers(workers):
    """Use scipy.fft with `workers` threads for the steps (large grids); None restores numpy.fft."""
    global _fft2, _ifft2
    if workers is None:
        _fft2, _ifft2 = np.fft.fft2, np.fft.ifft2
        return
    import scipy.fft as sf
    _fft2 = lambda a: sf.fft2(a, workers=workers)  # noqa: E731
    _ifft2 = lambda a: sf.ifft2(a, workers=workers)  # noqa: E731


def etdrk4_coeffs(L, dt, M=32):
    """benchmarks/benchmark_gray_scott.py:336-356 (complex128, real parts returned)."""
    r = np.exp(1j * np.pi * (np.arange(1, M + 1) - 0.5) / M)
    LR = dt * L[..., None] + r
    E = np.exp(dt * L)
    E2 = np.exp(dt * L / 2)
    Q = dt * np.mean((np.exp(LR / 2) - 1) / LR, axis=-1)
    f1 = dt * np.mean((-4 - LR + np.exp(LR) * (4 - 3 * LR + LR ** 2)) / LR ** 3, axis=-1)
    f2 = dt * np.mean((2 + LR + np.exp(LR) * (-2 + LR)) / LR ** 3, axis=-1)
    f3 = dt * np.mean((-4 - 3 * LR - LR ** 2 + np.exp(LR) * (4 - LR)) / LR ** 3, axis=-1)
    return tuple(np.real(x) for x in (E, E2, Q, f1, f2, f3))


def etdrk4_coeffs_separable(lam_y, lam_x, D, dt, M=32, workers=8):
    """etdrk4_coeffs(D * (lam_y[:, None] + lam_x[None, :]), dt) for large grids.

    Each table entry depends only on its value of L, so the contour means are
    evaluated once per distinct value (a separable symbol has few: the 1D
    symbols are even in k) in chunks on `workers` threads, then scattered back.
    Every distinct value goes through the same expression as etdrk4_coeffs, so
    the tables are identical to it.
    """
    from concurrent.futures import ThreadPoolExecutor
    L = D * (np.asarray(lam_y, dtype=np.float64)[:, None] + np.asarray(lam_x, dtype=np.float64)[None, :])
    vals, inv = np.unique(L, return_inverse=True)
    chunks = np.array_split(vals, max(1, len(vals) // 16384))
    with ThreadPoolExecutor(workers) as ex:
        parts = list(ex.map(lambda c: etdrk4_coeffs(c, dt, M), chunks))
    return tuple(np.concatenate([p[i] for p in parts])[inv].reshape(L.shape) for i in range(6))


def gs_nonlinear(u, v, F, k):
    """benchmark_gray_scott.py:376-380."""
    return -u * v * v + F * (1 - u), u * v * v - (F + k) * v


def etdrk4_step(u, v, cu, cv, F, k, f2_factor=1.0):
    """benchmark_gray_scott.py:369-417 (one coupled step); cu/cv = coefficient tuples.

    f2_factor=1 is the benchmark's update (f2 (N^a + N^b), line 415); 2 is the
    Cox-Matthews/Kassam-Trefethen update (2 f2 (N^a + N^b)).
    """
    fft2, ifft2 = _fft2, _ifft2
    Eu, E2u, Qu, f1u, f2u, f3u = cu
    Ev, E2v, Qv, f1v, f2v, f3v = cv
    uh, vh = fft2(u), fft2(v)
    nu, nv = gs_nonlinear(u, v, F, k)
    Nu, Nv = fft2(nu), fft2(nv)
    au, av = E2u * uh + Qu * Nu, E2v * vh + Qv * Nv
    ar, br_ = np.real(ifft2(au)), np.real(ifft2(av))
    nau, nav = gs_nonlinear(ar, br_, F, k)
    Nau, Nav = fft2(nau), fft2(nav)
    bu, bv = E2u * uh + Qu * Nau, E2v * vh + Qv * Nav
    bur, bvr = np.real(ifft2(bu)), np.real(ifft2(bv))
    nbu, nbv = gs_nonlinear(bur, bvr, F, k)
    Nbu, Nbv = fft2(nbu), fft2(nbv)
    cuh = E2u * au + Qu * (2 * Nbu - Nu)
    cvh = E2v * av + Qv * (2 * Nbv - Nv)
    cur, cvr = np.real(ifft2(cuh)), np.real(ifft2(cvh))
    ncu, ncv = gs_nonlinear(cur, cvr, F, k)
    Ncu, Ncv = fft2(ncu), fft2(ncv)
    un = Eu * uh + f1u * Nu + f2_factor * f2u * (Nau + Nbu) + f3u * Ncu
    vn = Ev * vh + f1v * Nv + f2_factor * f2v * (Nav + Nbv) + f3v * Ncv
    return np.real(ifft2(un)), np.real(ifft2(vn))


def etdrk4_gray_scott(u0, v0, lam, Du, Dv, F, k, dt, n_steps, f2_factor=1.0):
    """n_steps fixed steps from interior (ny, nx) fields; lam = Laplacian symbol (ny, nx)."""
    cu = etdrk4_coeffs(Du * lam, dt)
    cv = etdrk4_coeffs(Dv * lam, dt)
    u, v = np.array(u0, dtype=np.float64), np.array(v0, dtype=np.float64)
    for _ in range(n_steps):
        u, v = etdrk4_step(u, v, cu, cv, F, k, f2_factor)
    return u, v


def phi_functions(z):
    """phi_1..3 by their closed forms (moljax/core/fft_integrators.py:39-78), large |z|."""
    phi1 = np.expm1(z) / z
    phi2 = (np.expm1(z) - z) / z ** 2
    phi3 = (np.expm1(z) - z - z ** 2 / 2) / z ** 3
    return phi1, phi2, phi3
