"""Oracle: 1D tubular reactor, Crank-Nicolson (dense FP64 as the reference).

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restates two
reference discretisations of c_t = (1/Pe) c_zz - c_z - Da c:

* ``danckwerts_cn`` -- benchmarks/benchmark_reactor_vs_diffrax.py:40-138:
  N cells (dz = 1/N), FD Laplacian with the outlet Neumann row
  L[-1,-2] = 2 (40-48), upwind gradient with G[0,0] = 0 (51-57), Danckwerts
  inlet flux adv[0] = -(c0 - 1)/dz (86), semi-implicit CN
  c' = A^-1 (B c + dt (adv - Da c)), A = I - dt/(2Pe) L, B = I + dt/(2Pe) L;
* ``dirichlet_cn`` -- benchmarks/benchmark_method_comparison.py:56-160:
  N nodes (dz = 1/(N-1)), L = D2/Pe - D1 - Da I with row 0 zero (Dirichlet
  inlet) and the one-sided outlet row (96-100), fully implicit CN with
  A_lhs row 0 = e0 and rhs[0] = c_inlet (134-160), dense solve.
"""

from __future__ import annotations

import numpy as np


def danckwerts_cn(N, Pe, Da, dt, n_steps, c_init=1.0):
    dz = 1.0 / N
    L = (np.diag(-2.0 * np.ones(N)) + np.diag(np.ones(N - 1), 1) + np.diag(np.ones(N - 1), -1))
    L[-1, -1] = -2.0
    L[-1, -2] = 2.0
    L /= dz ** 2
    G = np.diag(np.ones(N)) + np.diag(-np.ones(N - 1), -1)
    G[0, 0] = 0.0
    G /= dz
    I = np.eye(N)
    A = I - 0.5 * dt / Pe * L
    B = I + 0.5 * dt / Pe * L
    Ainv = np.linalg.inv(A)
    c = np.full(N, float(c_init))
    for _ in range(n_steps):
        adv = -G @ c
        adv[0] = -(c[0] - 1.0) / dz
        c = Ainv @ (B @ c + dt * (adv - Da * c))
    return c


def danckwerts_full_cn(N, Pe, Da, dt, n_steps, c_init=0.0):
    """The Danckwerts discretisation of danckwerts_cn (benchmark_reactor_vs_diffrax.py:40-138:
    N cells, dz = 1/N, Neumann outlet row, inlet flux -(c0 - 1)/dz) advanced by the fully
    implicit Crank-Nicolson of benchmark_method_comparison.py:134-160: with M the whole
    operator (dispersion, upwind advection, reaction) and s = e0/dz the inlet source,
    (I - dt/2 M) c' = (I + dt/2 M) c + dt s.  Dense FP64."""
    dz = 1.0 / N
    L = (np.diag(-2.0 * np.ones(N)) + np.diag(np.ones(N - 1), 1) + np.diag(np.ones(N - 1), -1))
    L[-1, -1] = -2.0
    L[-1, -2] = 2.0
    L /= dz ** 2
    G = np.diag(np.ones(N)) + np.diag(-np.ones(N - 1), -1)
    G /= dz                      # row 0: c0/dz (the inlet flux without its source)
    M = L / Pe - G - Da * np.eye(N)
    s = np.zeros(N)
    s[0] = 1.0 / dz
    I = np.eye(N)
    A = I - 0.5 * dt * M
    B = I + 0.5 * dt * M
    Ainv = np.linalg.inv(A)
    c = np.full(N, float(c_init))
    for _ in range(n_steps):
        c = Ainv @ (B @ c + dt * s)
    return c


def dirichlet_system(N, Pe, Da):
    """benchmarks/benchmark_method_comparison.py:56-110 (the full operator L)."""
    dz = 1.0 / (N - 1)
    D2 = np.zeros((N, N))
    for i in range(1, N - 1):
        D2[i, i - 1], D2[i, i], D2[i, i + 1] = 1.0, -2.0, 1.0
    D2 /= dz ** 2
    D1 = np.zeros((N, N))
    for i in range(1, N):
        D1[i, i - 1], D1[i, i] = -1.0, 1.0
    D1 /= dz
    L = (1.0 / Pe) * D2 - D1 - Da * np.eye(N)
    L[0, :] = 0.0
    L[-1, :] = 0.0
    L[-1, -2] = (1.0 / Pe) / dz ** 2
    L[-1, -1] = -(1.0 / Pe) / dz ** 2 - 1.0 / dz - Da
    return L


def dirichlet_cn(N, Pe, Da, dt, n_steps, c_inlet=1.0, c_init=0.0):
    """benchmarks/benchmark_method_comparison.py:134-160 with c0 = 0, c0[0] = 1 (188-190)."""
    L = dirichlet_system(N, Pe, Da)
    I = np.eye(N)
    Al = I - 0.5 * dt * L
    Ar = I + 0.5 * dt * L
    Al[0, :] = 0.0
    Al[0, 0] = 1.0
    Ar[0, :] = 0.0
    c = np.full(N, float(c_init))
    c[0] = c_inlet
    for _ in range(n_steps):
        r = Ar @ c
        r[0] = c_inlet
        c = np.linalg.solve(Al, r)
    return c


def served_dt(N, t_final=5.0):
    """dt = min(10 dz, 0.05, t_final/100), dz = 1/(N-1) (benchmark_method_comparison.py:215-217)."""
    dz = 1.0 / (N - 1)
    dt = min(10 * dz, 0.05, t_final / 100)
    return dt, int(t_final / dt)
