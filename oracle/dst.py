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
