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


def implicit_step(u, u_prev, method, dt, dt_prev, dy, dx, a=1.0, b=1.0, c=1.0, restart=30,
                  newton_tol=1e-8, krylov_tol=1e-6, max_krylov=50, max_newton=10,
                  be_guess="euler"):
    """be_step / cn_step / bdf2_step (moljax/core/stepping.py:170-310) for the model above.

    method: "be", "cn" or "bdf2"; returns (u_new, converged, newton_iters, gmres_iters).
    """
    F = lambda y: vardiff_F(y, dy, dx, a, b, c)  # noqa: E731
    J = lambda y, v: vardiff_JF(y, v, dy, dx, a, b, c)  # noqa: E731
    if method == "be":
        a0, beta, cst = 1.0, dt, -u
    elif method == "cn":
        a0, beta, cst = 1.0, 0.5 * dt, -u - 0.5 * dt * F(u)
    else:
        a0, a1, a2, beta = bdf2_coeffs(dt, dt_prev)
        cst = a1 * u + a2 * u_prev
    if method == "bdf2":
        guess = 2 * u - u_prev
    else:
        guess = u + dt * F(u) if be_guess == "euler" else u.copy()
    Dbar = a + b * float(np.mean(u * u))
    res = lambda y: a0 * y + cst - beta * F(y)  # noqa: E731
    jvp = lambda y, v: a0 * v - beta * J(y, v)  # noqa: E731
    Mi = lambda r: dirichlet_helmholtz(r, dy, dx, a0, beta * Dbar)  # noqa: E731
    un, conv, it, li, rr = newton_krylov(res, jvp, guess, Mi, newton_tol, krylov_tol,
                                         max_newton=max_newton, restart=restart,
                                         max_krylov=max_krylov)
    return un, conv, it, li


def adaptive_integrate_implicit(u0, dy, dx, method, t0, t_end, dt0, atol=1e-6, rtol=1e-3,
                                safety=0.9, kI=0.7, kP=0.4, dt_min=1e-12, dt_max=1.0,
                                max_factor=5.0, min_factor=0.2, max_steps=10000,
                                save_every=1, a=1.0, b=1.0, c=1.0, be_guess="euler", **nk):
    """Implicit branch of adaptive_integrate (moljax/core/stepping.py:723-1021).

    Error: BE -> dt F(y_be); CN/BDF2 -> y_method - y_BE (BDF2 starts with BE while
    step_count < 1).  propose_dt (dt_policy.py:324-408): PI on accept, the reject
    formula otherwise, then implicit_robustness_dt (279-321, defaults: x0.5 when
    Newton did not converge, x1.2 capped at 1.0 when it converged in <= 3
    iterations, clip to [1e-12, 1]) and the final clamp to [dt_min, dt_max].
    Returns dict(t, u, t_hist, dt_hist, n_acc, n_rej, status, write_idx).
    """
    order = 1 if method == "be" else 2
    max_saves = max_steps // save_every + 1
    t_hist, dt_hist = np.zeros(max_saves), np.zeros(max_saves)
    t_hist[0] = t0
    nan_max = lambda x, y: x + y if (x != x or y != y) else max(x, y)  # noqa: E731
    nan_min = lambda x, y: x + y if (x != x or y != y) else min(x, y)  # noqa: E731
    clip = lambda x, lo, hi: nan_min(nan_max(x, lo), hi)  # noqa: E731
    t, u, u_prev, dt, dt_prev = float(t0), u0.copy(), u0.copy(), float(dt0), float(dt0)
    prev_err, step_count, write_idx, n_acc, n_rej, status = 1.0, 0, 1, 0, 0, 1
    log = []
    while status == 1 and t < t_end and write_idx < max_saves:
        dtc = nan_min(dt, t_end - t)
        if method == "be" or (method == "bdf2" and step_count < 1):
            un, conv, it, _ = implicit_step(u, u_prev, "be", dtc, dt_prev, dy, dx, a, b, c,
                                            be_guess=be_guess, **nk)
            err = dtc * vardiff_F(un, dy, dx, a, b, c)
        else:
            un, conv, it, _ = implicit_step(u, u_prev, method, dtc, dt_prev, dy, dx, a, b, c,
                                            be_guess=be_guess, **nk)
            ube, _, _, _ = implicit_step(u, u_prev, "be", dtc, dt_prev, dy, dx, a, b, c,
                                         be_guess=be_guess, **nk)
            err = un - ube
        q = err / (atol + rtol * np.abs(un))
        e = nan_max(float(np.sqrt(np.sum(q * q) / q.size)), 1e-10)
        finite = bool(np.all(np.isfinite(un)))
        accept = e <= 1.0 and finite and conv
        if e <= 1.0:
            fac = clip((1.0 / max(e, 1e-10)) ** (kI / order) * (max(prev_err, 1e-10) / max(e, 1e-10))
                       ** (kP / order) * safety, min_factor, max_factor)
            dt_a, pe_new = clip(dtc * fac, dt_min, dt_max), e
        else:
            fac = clip(safety * (1.0 / nan_max(e, 1.0)) ** (kI / order), min_factor, 1.0)
            dt_a, pe_new = clip(dtc * fac, dt_min, dt_max), prev_err
        dt_r = dt_a if conv else dt_a * 0.5
        if conv and it <= 3:
            dt_r = nan_min(dt_r * 1.2, 1.0)
        dt_new = clip(clip(dt_r, 1e-12, 1.0), dt_min, dt_max)
        log.append((t, dtc, e, conv, it, accept))
        if accept:
            if n_acc % save_every == 0:
                t_hist[write_idx] = t + dtc
                dt_hist[write_idx - 1] = dtc
                write_idx += 1
            t = t + dtc
            u_prev, u = u, un
            dt, dt_prev = dt_new, dtc
            step_count += 1
            prev_err = pe_new
            n_acc += 1
        else:
            dt = nan_max(dt_new * 0.5, dt_min)
            if dt <= dt_min * 1.1:
                status = 3
            n_rej += 1
        if not finite:
            status = 4
    if t >= t_end:
        status = 0
    elif write_idx >= max_saves:
        status = 2
    return dict(t=t, u=u, t_hist=t_hist, dt_hist=dt_hist, n_acc=n_acc, n_rej=n_rej,
                status=status, write_idx=write_idx, log=log)


def replay_implicit_controller(log, method, t0, t_end, dt0, safety=0.9, kI=0.7, kP=0.4,
                               dt_min=1e-12, dt_max=1.0, max_factor=5.0, min_factor=0.2):
    """Re-runs the accept/reject and dt logic of adaptive_integrate's implicit branch on a
    recorded attempt sequence (t, dt, err, converged, newton_iters, accepted) and returns the
    (t, dt, accepted) each attempt should have had (stepping.py:723-1021, dt_policy.py:178-408)."""
    order = 1 if method == "be" else 2
    nan_max = lambda x, y: x + y if (x != x or y != y) else max(x, y)  # noqa: E731
    nan_min = lambda x, y: x + y if (x != x or y != y) else min(x, y)  # noqa: E731
    clip = lambda x, lo, hi: nan_min(nan_max(x, lo), hi)  # noqa: E731
    t, dt, prev_err = float(t0), float(dt0), 1.0
    out = []
    for (_, _, e, conv, it, _) in log:
        dtc = nan_min(dt, t_end - t)
        accept = e <= 1.0 and bool(conv)
        out.append((t, dtc, accept))
        if e <= 1.0:
            fac = clip((1.0 / max(e, 1e-10)) ** (kI / order) * (max(prev_err, 1e-10) / max(e, 1e-10))
                       ** (kP / order) * safety, min_factor, max_factor)
            dt_a, pe_new = clip(dtc * fac, dt_min, dt_max), e
        else:
            fac = clip(safety * (1.0 / nan_max(e, 1.0)) ** (kI / order), min_factor, 1.0)
            dt_a, pe_new = clip(dtc * fac, dt_min, dt_max), prev_err
        dt_r = dt_a if conv else dt_a * 0.5
        if conv and it <= 3:
            dt_r = nan_min(dt_r * 1.2, 1.0)
        dt_new = clip(clip(dt_r, 1e-12, 1.0), dt_min, dt_max)
        if accept:
            t, dt, prev_err = t + dtc, dt_new, pe_new
        else:
            dt = nan_max(dt_new * 0.5, dt_min)
    return out


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
