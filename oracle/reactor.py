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


# --- penalty-BC RK4 (benchmarks/benchmark_tubular_reactor.py) ---------------------------

TUBULAR_BCS = ("danckwerts", "robin", "neumann")


def tubular_dt(N, Pe, t_final):
    """dt = min(0.5 dz, 0.25 Pe dz^2, 0.01), n_steps = int(t_final / dt), dz = 1/(N-1)
    (benchmark_tubular_reactor.py:254-256, 283-286)."""
    dz = 1.0 / (N - 1)
    dt = min(0.5 * dz, 0.25 * Pe * dz ** 2, 0.01)
    return dt, int(t_final / dt)


def tubular_rhs(c, N, Pe, Da, bc, c_in=1.0):
    """dc/dt of benchmark_tubular_reactor.py:57-160 on N nodes (dz = 1/(N-1)): the interior
    rows (1/Pe) D2 c - D1 c - Da c (D2 central with zero end rows, D1 central with one-sided
    end rows, 57-81), then the two end rows replaced by penalty relaxations 100 (target - c):
    Danckwerts inlet target (c_in + k c1) / (1 + k), k = (1/Pe)/dz (84-110); Robin with
    alpha_in = 1, beta_in = 1/Pe, alpha_out = 0, beta_out = 1 (113-144, 269); Neumann
    c1 / c_{N-2} (147-167).  Written out per row, in the reference's operation order."""
    dz = 1.0 / (N - 1)
    d2 = np.zeros_like(c)
    d2[1:-1] = (c[:-2] - 2.0 * c[1:-1] + c[2:]) / dz ** 2
    d1 = np.empty_like(c)
    d1[1:-1] = (-0.5 * c[:-2] + 0.5 * c[2:]) / dz
    d1[0] = (-c[0] + c[1]) / dz
    d1[-1] = (-c[-2] + c[-1]) / dz
    f = (1.0 / Pe) * d2 - d1 - Da * c
    if bc == "danckwerts":
        k = (1.0 / Pe) / dz
        f[0] = 100.0 * ((c_in + k * c[1]) / (1.0 + k) - c[0])
        f[-1] = 100.0 * (c[-2] - c[-1])
    elif bc == "robin":
        b_in, b_out = 1.0 / Pe, 1.0
        f[0] = 100.0 * ((c_in + b_in / dz * c[1]) / (1.0 + b_in / dz) - c[0])
        f[-1] = 100.0 * ((b_out / dz * c[-2]) / (0.0 + b_out / dz) - c[-1])
    elif bc == "neumann":
        f[0] = 100.0 * (c[1] - c[0])
        f[-1] = 100.0 * (c[-2] - c[-1])
    else:
        raise ValueError(bc)
    return f


def tubular_initial(N, bc):
    """Zeros (Danckwerts, Robin) or ones (Neumann) (benchmark_tubular_reactor.py:258-262)."""
    return np.ones(N) if bc == "neumann" else np.zeros(N)


def tubular_rk4_loop(N, Pe, Da, bc, dt, n_steps, c0=None):
    """Classical RK4 (benchmark_tubular_reactor.py:181-192), step by step."""
    c = tubular_initial(N, bc) if c0 is None else np.array(c0, dtype=np.float64)
    f = lambda y: tubular_rhs(y, N, Pe, Da, bc)
    for _ in range(n_steps):
        k1 = f(c)
        k2 = f(c + 0.5 * dt * k1)
        k3 = f(c + 0.5 * dt * k2)
        k4 = f(c + dt * k3)
        c = c + (dt / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
    return c


def tubular_rk4(N, Pe, Da, bc, dt, n_steps):
    """The same RK4 recurrence for long runs: the RHS is affine, f(c) = A c + b, so one step
    is c <- P c + q with P = I + hA + (hA)^2/2 + (hA)^3/6 + (hA)^4/24 and
    q = h (I + hA/2 + (hA)^2/6 + (hA)^3/24) b (exact algebra of the four stages); n steps are
    the n-th power of the affine map, by repeated squaring (FP64)."""
    I = np.eye(N)
    b = tubular_rhs(np.zeros(N), N, Pe, Da, bc)
    A = np.stack([tubular_rhs(I[:, j], N, Pe, Da, bc) - b for j in range(N)], axis=1)
    hA = dt * A
    hA2 = hA @ hA
    hA3 = hA2 @ hA
    P = I + hA + hA2 / 2 + hA3 / 6 + hA3 @ hA / 24
    q = dt * ((I + hA / 2 + hA2 / 6 + hA3 / 24) @ b)
    T = np.eye(N + 1)
    T[:N, :N] = P
    T[:N, N] = q
    R = np.eye(N + 1)
    n = int(n_steps)
    while n:
        if n & 1:
            R = T @ R
        T = T @ T
        n >>= 1
    c0 = np.append(tubular_initial(N, bc), 1.0)
    return (R @ c0)[:N]


def tubular_analytic_danckwerts(z, Pe, Da):
    """Steady state of the Danckwerts problem (benchmark_tubular_reactor.py:207-235):
    c = A e^{r1 z} + B e^{r2 z}, r = (Pe +- sqrt(Pe^2 + 4 Pe Da))/2."""
    disc = Pe ** 2 + 4 * Pe * Da
    r1 = (Pe + np.sqrt(disc)) / 2
    r2 = (Pe - np.sqrt(disc)) / 2
    M = np.array([[r1 / Pe - 1, r2 / Pe - 1], [r1 * np.exp(r1), r2 * np.exp(r2)]])
    A, B = np.linalg.solve(M, np.array([-1.0, 0.0]))
    return A * np.exp(r1 * z) + B * np.exp(r2 * z)


def tubular_summary(c, Pe, Da, bc, t_final):
    """conversion (1 - outlet, or the mean for Neumann), the max error against the
    analytic profile (the Danckwerts steady state, or e^{-Da t} for Neumann) and the outlet
    value (benchmark_tubular_reactor.py:263-268, 294-296)."""
    N = c.shape[-1]
    z = np.linspace(0, 1, N)
    ref = tubular_analytic_danckwerts(z, Pe, Da) if bc != "neumann" else np.exp(-Da * t_final) * np.ones(N)
    conv = 1.0 - c[-1] if bc != "neumann" else float(c.mean())
    return {"conversion": float(conv), "error": float(np.max(np.abs(c - ref))), "final_outlet_c": float(c[-1])}
