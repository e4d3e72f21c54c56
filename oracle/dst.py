"""Oracle: DST-I and the Dirichlet spectral solvers of moljax/core/fft_nonperiodic.py.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  NumPy FP64 restatement
of dst_I_fast / idst_I_fast (fft_nonperiodic.py:97-133: DST-I read off the
FFT of the odd extension of length 2(N+1)), laplacian_symbol_dirichlet
(140-162), solve_poisson_dirichlet (244-271), solve_helmholtz_dirichlet
(308-330) and etd1_dirichlet (360-398), all along the last axis.  Pinned by
the reference's own test assertions (tests/test_fft_nonperiodic.py:24-80) and
by scipy.fft.dst(type=1), which is twice this transform.
"""

from __future__ import annotations

import numpy as np


def dst_I_fast(x):
    """X[k] = sum_n x[n] sin(pi (k+1)(n+1)/(N+1)) along the last axis."""
    x = np.asarray(x, dtype=np.float64)
    N = x.shape[-1]
    z = np.zeros(x.shape[:-1] + (2 * (N + 1),))
    z[..., 1:N + 1] = x
    z[..., N + 2:] = -x[..., ::-1]
    return -0.5 * np.imag(np.fft.fft(z, axis=-1)[..., 1:N + 1])


def idst_I_fast(X):
    N = np.asarray(X).shape[-1]
    return dst_I_fast(X) * 2.0 / (N + 1)


def laplacian_symbol_dirichlet(N, dx):
    k = np.arange(1, N + 1, dtype=np.float64)
    return -4.0 / (dx * dx) * np.sin(np.pi * k / (2 * (N + 1))) ** 2


def solve_poisson_dirichlet(rhs, lam):
    return idst_I_fast(dst_I_fast(rhs) / lam)


def solve_helmholtz_dirichlet(rhs, lam, dt, D):
    return idst_I_fast(dst_I_fast(rhs) / (1.0 - dt * D * lam))


def etd1_dirichlet(u, N_u, eig, dt):
    z = dt * np.asarray(eig, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        phi1 = np.where(np.abs(z) < 1e-4, 1.0 + z / 2.0 + z ** 2 / 6.0, (np.exp(z) - 1.0) / z)
    return idst_I_fast(np.exp(z) * dst_I_fast(u) + dt * phi1 * dst_I_fast(N_u))


# ---------------------------------------------------------------- Neumann (DCT-II)
def dct2_ortho(x):
    """Orthonormal DCT-II along the last axis, written out from its definition
    (jax.scipy.fft.dct(x, type=2, norm='ortho'), scipy's convention): y[k] = f_k *
    2 sum_n x[n] cos(pi k (2n+1) / 2N), f_0 = sqrt(1/4N), f_k = sqrt(1/2N)."""
    x = np.asarray(x, dtype=np.float64)
    N = x.shape[-1]
    n = np.arange(N)
    C = 2.0 * np.cos(np.pi * np.outer(np.arange(N), 2 * n + 1) / (2 * N))
    f = np.full(N, np.sqrt(0.5 / N))
    f[0] = np.sqrt(0.25 / N)
    return (x @ C.T) * f


def idct2_ortho(X):
    """Inverse of dct2_ortho (DCT-III): x[n] = w0 X0 + sum_k wk Xk cos(pi k (2n+1) / 2N)."""
    X = np.asarray(X, dtype=np.float64)
    N = X.shape[-1]
    k = np.arange(N)
    C = np.cos(np.pi * np.outer(2 * np.arange(N) + 1, k) / (2 * N))
    w = np.full(N, np.sqrt(2.0 / N))
    w[0] = np.sqrt(1.0 / N)
    return (X * w) @ C.T


def laplacian_symbol_neumann(N, dx):
    k = np.arange(N, dtype=np.float64)
    return -4.0 / (dx * dx) * np.sin(np.pi * k / (2 * N)) ** 2


def solve_poisson_neumann(rhs, lam):
    X = dct2_ortho(rhs)
    with np.errstate(divide="ignore", invalid="ignore"):
        U = np.where(np.abs(lam) < 1e-14, 0.0, X / lam)
    return idct2_ortho(U)


def solve_helmholtz_neumann(rhs, lam, dt, D):
    return idct2_ortho(dct2_ortho(rhs) / (1.0 - dt * D * lam))


def etd1_neumann(u, N_u, eig, dt):
    z = dt * np.asarray(eig, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        phi1 = np.where(np.abs(z) < 1e-4, 1.0 + z / 2.0 + z ** 2 / 6.0, (np.exp(z) - 1.0) / z)
    return idct2_ortho(np.exp(z) * dct2_ortho(u) + dt * phi1 * dct2_ortho(N_u))
