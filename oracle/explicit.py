"""Oracle: explicit Runge-Kutta steps, step doubling and the explicit branch of
adaptive_integrate, for reaction-advection-diffusion models with any ghost BCs.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  NumPy FP64
restatement of moljax/core/stepping.py:64-163 (euler_step, ssprk3_step,
rk4_step), 566-608 (step doubling), 648-682 (step_explicit_with_error) and
the explicit path of adaptive_integrate (723-1021) with propose_dt
(dt_policy.py:324-408) and heisenberg_cfl_dt (104-175).  The model right-hand
side is MOLModel.rhs (model.py:100-118): BCs first, then
D Lap(u) - vx du/dx - vy du/dy (operators.py:200-322) plus the reaction
(operators.py:644-705).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Dict, Optional

import numpy as np

from oracle import mol
from oracle.imex import (CFLParams, PIDParams, SUCCESS, RUNNING, MAX_STEPS_REACHED, DT_TOO_SMALL,
                         NON_FINITE_VALUES, AdaptiveResult, pid_controller_dt, handle_rejected_step)

ORDER = {0: 1, 1: 3, 2: 4}  # compute_error_order (dt_policy.py:411-423): Euler, SSPRK3, RK4


@dataclass
class ExplicitModel:
    grid: object
    kinds: Dict[str, int]
    D: Dict[str, float]
    values: Dict[str, Dict[str, float]] = field(default_factory=dict)
    reaction: Optional[Callable] = None
    vx: float = 0.0
    vy: float = 0.0
    advection: Optional[str] = None  # None, "upwind", "central"
    params: Dict[str, float] = field(default_factory=dict)

    def apply_bcs(self, y):
        return {k: mol.bc_2d(f, self.grid, self.kinds[k], self.values.get(k)) for k, f in y.items()}

    def rhs(self, y):
        y = self.apply_bcs(y)
        g = self.grid
        out = {}
        for k, f in y.items():
            r = self.D.get(k, 0.0) * mol.laplacian_2d(f, g)
            if self.advection == "upwind":
                r = r - self.vx * mol.d1_upwind_2d(f, self.vx, g, 1) - self.vy * mol.d1_upwind_2d(f, self.vy, g, 0)
            elif self.advection == "central":
                r = r - self.vx * _central(f, g, 1) - self.vy * _central(f, g, 0)
            out[k] = r
        if self.reaction is not None:
            R = self.reaction(y)
            s = g.interior_slice
            for k in out:
                out[k][s] = out[k][s] + R[k][s]
        return out


def _central(f, g, axis):
    """d1_central_2d (operators.py:155-197): (f[+1] - f[-1]) / (2 d) on the interior."""
    n, nx, ny = g.n_ghost, g.nx, g.ny
    out = np.zeros_like(f, dtype=np.float64)
    if axis == 0:
        out[n:n + ny, n:n + nx] = (f[n + 1:n + ny + 1, n:n + nx] - f[n - 1:n + ny - 1, n:n + nx]) / (2 * g.dy)
    else:
        out[n:n + ny, n:n + nx] = (f[n:n + ny, n + 1:n + nx + 1] - f[n:n + ny, n - 1:n + nx - 1]) / (2 * g.dx)
    return out


def _axpy(y, a, x):
    return {k: y[k] + a * x[k] for k in y}


def euler_step(model, y, dt):
    return _axpy(y, dt, model.rhs(y))


def ssprk3_step(model, y, dt):
    y1 = _axpy(y, dt, model.rhs(y))
    F1 = model.rhs(y1)
    y2 = {k: 0.75 * y[k] + 0.25 * y1[k] + 0.25 * dt * F1[k] for k in y}
    F2 = model.rhs(y2)
    return {k: y[k] / 3.0 + 2.0 / 3.0 * y2[k] + 2.0 / 3.0 * dt * F2[k] for k in y}


def rk4_step(model, y, dt):
    k1 = model.rhs(y)
    k2 = model.rhs(_axpy(y, 0.5 * dt, k1))
    k3 = model.rhs(_axpy(y, 0.5 * dt, k2))
    k4 = model.rhs(_axpy(y, dt, k3))
    return {k: y[k] + dt / 6.0 * (k1[k] + 2.0 * k2[k] + 2.0 * k3[k] + k4[k]) for k in y}


STEPS = {0: euler_step, 1: ssprk3_step, 2: rk4_step}


def step_explicit_with_error(model, y, dt, method):
    """Step doubling: (y_half2, y_half2 - y_full)."""
    step = STEPS[method]
    y_full = step(model, y, dt)
    y_h2 = step(model, step(model, y, 0.5 * dt), 0.5 * dt)
    return y_h2, {k: y_h2[k] - y_full[k] for k in y}


def heisenberg_cfl_dt(grid, params, cfl):
    dx, dx2 = min(grid.dx, grid.dy), min(grid.dx, grid.dy) ** 2
    dt = cfl.dt_max
    v = abs(params.get("vx", 0.0)) + abs(params.get("vy", 0.0))
    dt = min(dt, cfl.cfl_advection * dx / v if v > 1e-14 else cfl.dt_max)
    Dm = max(params.get("D", 0.0), params.get("Du", 0.0), params.get("Dv", 0.0))
    dt = min(dt, cfl.cfl_diffusion * dx2 / Dm if Dm > 1e-14 else cfl.dt_max)
    return min(max(cfl.safety * dt, cfl.dt_min), cfl.dt_max)


def adaptive_integrate_explicit(model, y0, t0, t_end, dt0, method, max_steps=10000, cfl=None,
                                pid=None, save_every=1, max_attempts=None):
    cfl = cfl or CFLParams()
    pid = pid or PIDParams()
    order = ORDER[method]
    grid = model.grid
    dt_cfl = heisenberg_cfl_dt(grid, model.params, cfl)
    dt = min(float(dt0), dt_cfl)
    max_saves = max_steps // save_every + 1
    t_hist, dt_hist = np.zeros(max_saves), np.zeros(max_saves)
    t_hist[0] = t0
    t, y, prev_err = float(t0), y0, 1.0
    write_idx, n_acc, n_rej, status, attempts = 1, 0, 0, RUNNING, 0
    while status == RUNNING and t < t_end and write_idx < max_saves:
        if max_attempts is not None and attempts >= max_attempts:
            break
        attempts += 1
        dtc = min(dt, t_end - t)
        y_new, err = step_explicit_with_error(model, y, dtc, method)
        e = max(mol.scaled_error_norm(err, y_new, grid, pid.atol, pid.rtol), 1e-10)
        finite = mol.is_finite(y_new)
        accept = e <= 1.0 and finite
        if e <= 1.0:
            dt_a, pe_new = pid_controller_dt(dtc, e, prev_err, pid, order)
        else:
            dt_a, pe_new = handle_rejected_step(dtc, e, pid, order), prev_err
        dt_new = min(max(min(dt_a, dt_cfl), pid.dt_min), pid.dt_max)
        if accept:
            if n_acc % save_every == 0:
                t_hist[write_idx] = t + dtc
                dt_hist[write_idx - 1] = dtc
                write_idx += 1
            t, y, dt, prev_err = t + dtc, y_new, dt_new, pe_new
            n_acc += 1
        else:
            dt = max(dt_new * 0.5, pid.dt_min)
            if dt <= pid.dt_min * 1.1:
                status = DT_TOO_SMALL
            n_rej += 1
        if not finite:
            status = NON_FINITE_VALUES
    if t >= t_end:
        status = SUCCESS
    elif write_idx >= max_saves:
        status = MAX_STEPS_REACHED
    return AdaptiveResult(t, y, t_hist, None, dt_hist, write_idx, n_acc, n_rej, status)


def fft_advdiff_inverse(r, grid, dt, D, vx, vy):
    """FFTAdvectionDiffusionPreconditioner (moljax/core/preconditioners.py:297-420) on an
    interior field: real(ifft2(fft2(r) / (1 - dt (D lam - i (vx kx + vy ky))))), lam the
    periodic FD symbol, kx, ky = 2 pi fftfreq; |denominator| < 1e-14 -> 1e-14."""
    lam = mol.fd_symbol_2d(grid.ny, grid.nx, grid.dy, grid.dx)
    kx = 2 * np.pi * np.fft.fftfreq(grid.nx, d=grid.dx)[None, :]
    ky = 2 * np.pi * np.fft.fftfreq(grid.ny, d=grid.dy)[:, None]
    den = 1.0 - dt * (D * lam - 1j * (vx * kx + vy * ky))
    den = np.where(np.abs(den) < 1e-14, 1e-14, den)
    return np.real(np.fft.ifft2(np.fft.fft2(r) / den))


def mass_action(species, reactions=(), linear=None, source=None):
    """Reaction callable (padded state -> rates) of a mass-action network: for each
    species source + sum_j linear[(s, j)] c_j + sum_r (products - reactants)_s rate_r
    prod c^order (the native network of make_kinetics_op, restated in NumPy)."""
    def R(y):
        out = {}
        for s in species:
            acc = np.zeros_like(y[s], dtype=np.float64) + (source or {}).get(s, 0.0)
            for (t, j), kv in (linear or {}).items():
                if t == s:
                    acc = acc + kv * y[j]
            out[s] = acc
        for rate, reac, prod in reactions:
            w = float(rate)
            for j, o in reac.items():
                w = w * y[j] ** int(o)
            for s in species:
                nu = prod.get(s, 0) - reac.get(s, 0)
                if nu:
                    out[s] = out[s] + nu * w
        return out
    return R
