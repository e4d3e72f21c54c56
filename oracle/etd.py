"""Oracle: ETD1, ETD2 and the library ETDRK4 for u_t = L u + N(u) on periodic grids.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  NumPy FP64 restatement
of moljax/core/fft_integrators.py: the phi functions with their Taylor switch
(39-78), _etdrk4_coefficients (81-116), etd1_step (119-175), etd2_step
(178-249), etdrk4_step (252-341, one field at a time), etd_integrate (344-393)
and diffusion_only_etd1 (513-542).  ``coupled=True`` evaluates the later
ETDRK4 stages on all fields together (the Gray-Scott pair), where the library
calls nonlinear_rhs with one field at a time.

Fields are 1D (n,) or 2D (ny, nx) arrays; ``lam`` maps each field name to its
operator eigenvalues D * symbol in numpy FFT order (shape of the field).
"""

from __future__ import annotations

import numpy as np


def phi1(z):
    """fft_integrators.py:39-52."""
    z = np.asarray(z, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        direct = (np.exp(z) - 1.0) / z
    return np.where(np.abs(z) < 1e-4, 1.0 + z / 2.0 + z ** 2 / 6.0 + z ** 3 / 24.0, direct)


def phi2(z):
    """fft_integrators.py:55-65."""
    z = np.asarray(z, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        direct = (np.exp(z) - 1.0 - z) / (z * z)
    return np.where(np.abs(z) < 1e-4, 0.5 + z / 6.0 + z ** 2 / 24.0 + z ** 3 / 120.0, direct)


def phi3(z):
    """fft_integrators.py:68-78."""
    z = np.asarray(z, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        direct = (np.exp(z) - 1.0 - z - z ** 2 / 2.0) / (z ** 3)
    return np.where(np.abs(z) < 1e-4, 1.0 / 6.0 + z / 24.0 + z ** 2 / 120.0 + z ** 3 / 720.0, direct)


def etdrk4_coefficients(z):
    """fft_integrators.py:81-116: (E, E2, phi1(z/2), phi1(z), b1, b2, b3, b4)."""
    p1, p2, p3 = phi1(z), phi2(z), phi3(z)
    b1 = p1 - 3 * p2 + 4 * p3
    b2 = 2 * p2 - 4 * p3
    b4 = -p2 + 4 * p3
    return np.exp(z), np.exp(z / 2.0), phi1(z / 2.0), p1, b1, b2, b2, b4


def _fft(u):
    return np.fft.fft(u) if u.ndim == 1 else np.fft.fft2(u)


def _ifft(u):
    return np.real(np.fft.ifft(u) if u.ndim == 1 else np.fft.ifft2(u))


def etd1_step(state, dt, lam, nonlinear):
    """fft_integrators.py:119-175: exp(z) u^ + dt phi1(z) N^; no operator -> Euler."""
    Nn = nonlinear(state)
    out = {}
    for k, u in state.items():
        if k in lam:
            z = dt * lam[k]
            out[k] = _ifft(np.exp(z) * _fft(u) + dt * phi1(z) * _fft(Nn[k]))
        else:
            out[k] = u + dt * Nn[k]
    return out


def etd2_step(state, dt, lam, nonlinear, N_prev=None):
    """fft_integrators.py:178-249: returns (new_state, N(state)); ETD1 without N_prev."""
    Nc = nonlinear(state)
    if N_prev is None:
        return etd1_step(state, dt, lam, nonlinear), Nc
    out = {}
    for k, u in state.items():
        if k in lam:
            z = dt * lam[k]
            Nh, Nph = _fft(Nc[k]), _fft(N_prev[k])
            out[k] = _ifft(np.exp(z) * _fft(u) + dt * phi1(z) * Nh + dt * phi2(z) * (Nh - Nph))
        else:
            out[k] = u + dt * (1.5 * Nc[k] - 0.5 * N_prev[k])
    return out, Nc


def etdrk4_step(state, dt, lam, nonlinear, coupled=False):
    """fft_integrators.py:252-341 with the phi coefficients.  ``coupled`` evaluates
    N(a), N(b), N(c) on all fields at once (needed for Gray-Scott); otherwise field
    by field as the library does (311, 319, 327)."""
    Nn = nonlinear(state)
    names = list(state)
    C = {k: etdrk4_coefficients(dt * lam[k]) for k in names}
    uh = {k: _fft(state[k]) for k in names}
    Nnh = {k: _fft(Nn[k]) for k in names}

    def stage_N(fields):
        if coupled:
            return nonlinear(fields)
        return {k: nonlinear({k: fields[k]})[k] for k in fields}

    ah = {k: C[k][1] * uh[k] + (dt / 2) * C[k][2] * Nnh[k] for k in names}
    Na = stage_N({k: _ifft(ah[k]) for k in names})
    Nah = {k: _fft(Na[k]) for k in names}
    bh = {k: C[k][1] * uh[k] + (dt / 2) * C[k][2] * Nah[k] for k in names}
    Nb = stage_N({k: _ifft(bh[k]) for k in names})
    Nbh = {k: _fft(Nb[k]) for k in names}
    ch = {k: C[k][1] * ah[k] + (dt / 2) * C[k][2] * (2 * Nbh[k] - Nnh[k]) for k in names}
    Nc = stage_N({k: _ifft(ch[k]) for k in names})
    Nch = {k: _fft(Nc[k]) for k in names}
    out = {}
    for k in names:
        E, _, _, _, b1, b2, _, b4 = C[k]
        out[k] = _ifft(E * uh[k] + dt * (b1 * Nnh[k] + b2 * (Nah[k] + Nbh[k]) + b4 * Nch[k]))
    return out


def etd_integrate(u0, t_span, dt, lam, nonlinear, method="etd1", save_every=1, coupled=False):
    """fft_integrators.py:344-393: n_steps = int((t_end - t_start) / dt)."""
    t0, t1 = t_span
    n_steps = int((t1 - t0) / dt)
    t_hist, hist = [t0], [u0]
    state, t, N_prev = u0, t0, None
    for step in range(n_steps):
        if method == "etd1":
            state = etd1_step(state, dt, lam, nonlinear)
        elif method == "etd2":
            state, N_prev = etd2_step(state, dt, lam, nonlinear, N_prev)
        elif method == "etdrk4":
            state = etdrk4_step(state, dt, lam, nonlinear, coupled)
        else:
            raise ValueError(method)
        t += dt
        if (step + 1) % save_every == 0:
            t_hist.append(t)
            hist.append(state)
    return np.array(t_hist), hist


def diffusion_only_etd1(u0, t_end, dt, lam):
    """fft_integrators.py:513-542: max(1, int(t_end/dt)) exact exponential steps."""
    n = max(1, int(t_end / dt))
    h = t_end / n
    u = u0
    for _ in range(n):
        u = _ifft(np.exp(h * lam) * _fft(u))
    return u


def fd_symbol_1d(n, dx):
    """Periodic second-order FD Laplacian symbol (2 cos(k dx) - 2) / dx^2, numpy order."""
    k = 2 * np.pi * np.fft.fftfreq(n, d=dx)
    return (2.0 * np.cos(k * dx) - 2.0) / dx ** 2


def logistic(alpha):
    """alpha u (1 - u) on every field (tests/test_fft_operators.py:533-535)."""
    return lambda s: {k: alpha * v * (1 - v) for k, v in s.items()}


def gray_scott(F, k):
    """Coupled Gray-Scott reaction terms (operators.py:655-667)."""
    def N(s):
        u, v = s["u"], s["v"]
        uvv = u * v * v
        return {"u": -uvv + F * (1 - u), "v": uvv - (F + k) * v}
    return N


def zero(s):
    return {k: np.zeros_like(v) for k, v in s.items()}


def adaptive_etd(u0, t0, t_end, dt0, lam, nonlinear, method="etdrk4", pid=None, max_steps=10000,
                 save_every=1, coupled=False, max_attempts=None):
    """Adaptive ETD1 / ETDRK4 by step doubling: the accept/reject flow of the explicit
    branch of adaptive_integrate (moljax/core/stepping.py:723-1021: y_half2 - y_full as the
    error, scaled_error_norm, PI controller with compute_error_order, halving after a
    reject, DT_TOO_SMALL / NON_FINITE_VALUES / MAX_STEPS_REACHED) without a CFL limit
    (the linear part is integrated exactly).  Returns an oracle.imex.AdaptiveResult."""
    from oracle import imex as OI
    pid = pid or OI.PIDParams()
    order = {"etd1": 1, "etdrk4": 4}[method]

    def step(y, h):
        if method == "etd1":
            return etd1_step(y, h, lam, nonlinear)
        return etdrk4_step(y, h, lam, nonlinear, coupled)

    max_saves = max_steps // save_every + 1
    t_hist, dt_hist = np.zeros(max_saves), np.zeros(max_saves)
    t_hist[0] = t0
    t, y, dt, prev_err = float(t0), u0, float(dt0), 1.0
    write_idx, n_acc, n_rej, status, attempts = 1, 0, 0, OI.RUNNING, 0
    names = list(u0)
    while status == OI.RUNNING and t < t_end and write_idx < max_saves:
        if max_attempts is not None and attempts >= max_attempts:
            break
        attempts += 1
        dtc = min(dt, t_end - t)
        y_full = step(y, dtc)
        y_h = step(step(y, 0.5 * dtc), 0.5 * dtc)
        err = np.stack([y_h[k] - y_full[k] for k in names])
        yn = np.stack([y_h[k] for k in names])
        finite = bool(np.all(np.isfinite(yn)))
        e = max(float(np.sqrt(np.mean((err / (pid.atol + pid.rtol * np.abs(yn))) ** 2))), 1e-10)
        if e <= 1.0:
            dt_a, pe_new = OI.pid_controller_dt(dtc, e, prev_err, pid, order)
        else:
            dt_a, pe_new = OI.handle_rejected_step(dtc, e, pid, order), prev_err
        dt_new = min(max(dt_a, pid.dt_min), pid.dt_max)
        if e <= 1.0 and finite:
            if n_acc % save_every == 0:
                t_hist[write_idx] = t + dtc
                dt_hist[write_idx - 1] = dtc
                write_idx += 1
            t, y, dt, prev_err = t + dtc, y_h, dt_new, pe_new
            n_acc += 1
        else:
            dt = max(dt_new * 0.5, pid.dt_min)
            if dt <= pid.dt_min * 1.1:
                status = OI.DT_TOO_SMALL
            n_rej += 1
        if not finite:
            status = OI.NON_FINITE_VALUES
    if t >= t_end:
        status = OI.SUCCESS
    elif write_idx >= max_saves:
        status = OI.MAX_STEPS_REACHED
    return OI.AdaptiveResult(t, y, t_hist, None, dt_hist, write_idx, n_acc, n_rej, status)
