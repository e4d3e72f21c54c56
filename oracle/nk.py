"""Oracle: Newton-Krylov with left-preconditioned restarted GMRES, BE/CN/BDF2
residuals, and the nonlinear diffusion-reaction model of the NK benchmark
configuration.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  Restates
moljax/core/newton_krylov.py:171-448 (Newton loop with convergence evaluated
before the update, 3-try backtracking with the 1 - 1e-4 alpha decrease test,
full damped step when no try is accepted) and the residual builders.  The
Krylov solver is a textbook restarted GMRES (modified Gram-Schmidt, Givens),
following the hand-written Arnoldi of benchmarks/sisc/bench_reaction_dominant.py:78-138;
jax.scipy.sparse.linalg.gmres itself is not available here, so GMRES iteration
counts are not pinned -- parity is on the Newton solution and residual.

Model (the 512^2 NK configuration; not a reference model): interior unknowns u
on a cell-centred grid with homogeneous Dirichlet ghosts (ghost = -neighbour,
moljax/core/bc.py:218-260), F(u) = div((a + b u^2) grad u) - c u^3 with the
face-averaged conservative flux of apply_variable_diffusion_2d
(moljax/core/variable_coeff.py:232-287) and D evaluated on the ghost-filled u.
"""

from __future__ import annotations

import numpy as np

from oracle import mol


def dirichlet_pad(u):
    """Interior (ny, nx) -> padded with homogeneous Dirichlet ghosts (x first, then y)."""
    p = np.zeros((u.shape[0] + 2, u.shape[1] + 2))
    p[1:-1, 1:-1] = u
    p[:, 0] = -p[:, 1]
    p[:, -1] = -p[:, -2]
    p[0, :] = -p[1, :]
    p[-1, :] = -p[-2, :]
    return p


def vardiff_F(u, dy, dx, a=1.0, b=1.0, c=1.0):
    """div((a + b u^2) grad u) - c u^3 on the interior (variable_coeff.py:232-287)."""
    p = dirichlet_pad(u)
    D = a + b * p * p
    C = slice(1, -1)
    dxp = 0.5 * (D[C, C] + D[C, 2:]) * (p[C, 2:] - p[C, C])
    dxm = 0.5 * (D[C, C] + D[C, :-2]) * (p[C, C] - p[C, :-2])
    dyp = 0.5 * (D[C, C] + D[2:, C]) * (p[2:, C] - p[C, C])
    dym = 0.5 * (D[C, C] + D[:-2, C]) * (p[C, C] - p[:-2, C])
    return (dxp - dxm) / dx ** 2 + (dyp - dym) / dy ** 2 - c * u ** 3


def vardiff_JF(u, v, dy, dx, a=1.0, b=1.0, c=1.0):
    """Directional derivative dF(u)[v] written out by hand."""
    p, q = dirichlet_pad(u), dirichlet_pad(v)
    D = a + b * p * p
    dD = 2.0 * b * p * q
    C = slice(1, -1)

    def flux(Dc, Dn, pc, pn, dDc, dDn, qc, qn):
        return 0.5 * (Dc + Dn) * (qn - qc) + 0.5 * (dDc + dDn) * (pn - pc)

    fxp = flux(D[C, C], D[C, 2:], p[C, C], p[C, 2:], dD[C, C], dD[C, 2:], q[C, C], q[C, 2:])
    fxm = flux(D[C, :-2], D[C, C], p[C, :-2], p[C, C], dD[C, :-2], dD[C, C], q[C, :-2], q[C, C])
    fyp = flux(D[C, C], D[2:, C], p[C, C], p[2:, C], dD[C, C], dD[2:, C], q[C, C], q[2:, C])
    fym = flux(D[:-2, C], D[C, C], p[:-2, C], p[C, C], dD[:-2, C], dD[C, C], q[:-2, C], q[C, C])
    return (fxp - fxm) / dx ** 2 + (fyp - fym) / dy ** 2 - 3.0 * c * u * u * v


def dirichlet_helmholtz(r, dy, dx, alpha, kappa):
    """(alpha I - kappa Lap_D)^-1 r, Lap_D the cell-centred Dirichlet 5-point Laplacian.

    Exact through the odd extension to a (2ny, 2nx) periodic box, where the
    periodic FD Laplacian restricted to the first quadrant equals Lap_D
    (DST-II diagonalisation; eigenvalues -4/d^2 sin^2(pi k / 2N)).
    """
    ny, nx = r.shape
    e = np.zeros((2 * ny, 2 * nx))
    e[:ny, :nx] = r
    e[:ny, nx:] = -r[:, ::-1]
    e[ny:, :] = -e[:ny, :][::-1, :]
    lam = mol.fd_symbol_2d(2 * ny, 2 * nx, dy, dx)
    out = np.fft.ifft2(np.fft.fft2(e) / (alpha - kappa * lam)).real
    return out[:ny, :nx]


def gmres(matvec, b, x0, tol, restart, maxiter, M=None):
    """Left-preconditioned restarted GMRES (MGS Arnoldi, Givens); returns (x, iterations).

    Stops when the preconditioned residual <= tol * ||M b||; maxiter counts restart cycles
    (the jax.scipy convention).
    """
    Mf = (lambda v: v) if M is None else M
    bp = Mf(b)
    bnorm = np.linalg.norm(bp)
    x = x0.copy()
    its = 0
    if bnorm == 0.0:
        return x, 0
    for _ in range(maxiter):
        r = Mf(b - matvec(x))
        beta = np.linalg.norm(r)
        if beta <= tol * bnorm:
            break
        V = [r / beta]
        H = np.zeros((restart + 1, restart))
        cs, sn = np.zeros(restart), np.zeros(restart)
        g = np.zeros(restart + 1)
        g[0] = beta
        k_used = 0
        for j in range(restart):
            w = Mf(matvec(V[j]))
            for i in range(j + 1):
                H[i, j] = np.vdot(V[i], w)
                w = w - H[i, j] * V[i]
            hn = np.linalg.norm(w)
            H[j + 1, j] = hn
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            den = np.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = H[j, j] / den, H[j + 1, j] / den
            H[j, j] = den
            H[j + 1, j] = 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            its += 1
            k_used = j + 1
            if abs(g[j + 1]) <= tol * bnorm or hn == 0.0:
                break
            V.append(w / hn)
        y = np.linalg.solve(np.triu(H[:k_used, :k_used]), g[:k_used])
        x = x + sum(y[i] * V[i] for i in range(k_used))
        if abs(g[k_used]) <= tol * bnorm:
            break
    return x, its


def newton_krylov(residual, jvp, x0, M, newton_tol=1e-8, krylov_tol=1e-6, max_newton=10,
                  restart=20, max_krylov=50, damping=1.0, backtrack=0.5, max_backtrack=3,
                  min_dec=1e-4):
    """moljax/core/newton_krylov.py:171-359 -> (x, converged, newton_iters, gmres_iters, res)."""
    x = x0.copy()
    r0 = np.linalg.norm(residual(x))
    converged = r0 < newton_tol
    res = r0
    it = lits = 0
    while it < max_newton and not converged:
        r = residual(x)
        rn = np.linalg.norm(r)
        converged = rn < newton_tol
        dx, li = gmres(lambda v: jvp(x, v), -r, np.zeros_like(r), krylov_tol, restart, max_krylov, M)
        lits += li
        alpha, xb, rb, acc = damping, x, rn, False
        for _ in range(max_backtrack):
            if acc:
                break
            xn = xb + alpha * dx
            rnn = np.linalg.norm(residual(xn))
            if rnn < (1.0 - min_dec * alpha) * rb:
                xb, rb, acc = xn, rnn, True
            else:
                alpha *= backtrack
        x = xb if acc else x + damping * dx
        res = rb
        it += 1
    return x, converged, it, lits, res


def bdf2_coeffs(dt, dt_prev):
    """moljax/core/newton_krylov.py:433-437."""
    om = dt / dt_prev
    return (1 + 2 * om) / (1 + om), -(1 + om), om ** 2 / (1 + om), dt * (1 + om) / (1 + 2 * om)


def bdf2_integrate(u0, dy, dx, dt, n_steps, a=1.0, b=1.0, c=1.0, restart=30, newton_tol=1e-8,
                   krylov_tol=1e-6, max_krylov=50, be_guess="euler"):
    """Fixed-dt BDF2 with a BE first step (stepping.py:1077-1139 with bdf2_step 263-310).

    Preconditioner: (alpha0 I - beta Dbar Lap_D)^-1 with Dbar = a + b mean(u^2).
    Returns (u, stats list of (newton_iters, gmres_iters, converged)).
    be_guess: "euler" (the reference's be_step guess) or "previous" (y_n).
    """
    F = lambda u: vardiff_F(u, dy, dx, a, b, c)  # noqa: E731
    J = lambda u, v: vardiff_JF(u, v, dy, dx, a, b, c)  # noqa: E731
    u_prev, u = u0.copy(), u0.copy()
    stats = []
    for s in range(n_steps):
        if s == 0:   # BE: R = y - y_n - dt F(y), guess = explicit Euler
            a0, a1, a2, beta = 1.0, -1.0, 0.0, dt
            # be_step's guess is an explicit Euler step (stepping.py:195-196);
            # be_guess="previous" starts Newton from y_n instead
            guess = u + dt * F(u) if be_guess == "euler" else u.copy()
        else:
            a0, a1, a2, beta = bdf2_coeffs(dt, dt)
            guess = 2 * u - u_prev
        cst = a1 * u + a2 * u_prev
        Dbar = a + b * float(np.mean(u * u))
        res = lambda y: a0 * y + cst - beta * F(y)  # noqa: E731
        jvp = lambda y, v: a0 * v - beta * J(y, v)  # noqa: E731
        Mi = lambda r: dirichlet_helmholtz(r, dy, dx, a0, beta * Dbar)  # noqa: E731
        un, conv, it, li, rr = newton_krylov(res, jvp, guess, Mi, newton_tol, krylov_tol,
                                             restart=restart, max_krylov=max_krylov)
        stats.append((it, li, conv))
        u_prev, u = u, un
    return u, stats


def gaussians_ic(n, seed=4, count=8):
    """Seeded sum of 8 Gaussians on [0,1]^2 cell centres: A~U[0,1], w~U[0.02,0.1], c~U[0,1]^2."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    u = np.zeros((n, n))
    for _ in range(count):
        A = rng.uniform(0.0, 1.0)
        w = rng.uniform(0.02, 0.1)
        cx, cy = rng.uniform(0.0, 1.0, 2)
        u += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    return u
