"""Oracle: IMEX-Strang / IMEX-Euler steps, step doubling, PI controller and the
adaptive IMEX driver.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  NumPy FP64
restatement of moljax/core/stepping.py and moljax/core/dt_policy.py.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Dict

import numpy as np

from oracle import mol

# moljax/core/utils.py:265-272
SUCCESS, RUNNING, MAX_STEPS_REACHED, DT_TOO_SMALL, NON_FINITE_VALUES, NK_FAILED = range(6)


@dataclass(frozen=True)
class CFLParams:
    """moljax/core/dt_policy.py:28-46."""
    safety: float = 0.9
    dt_min: float = 1e-12
    dt_max: float = 1.0
    cfl_advection: float = 0.5
    cfl_diffusion: float = 0.25
    cfl_wave: float = 0.5


@dataclass(frozen=True)
class PIDParams:
    """moljax/core/dt_policy.py:49-78."""
    safety: float = 0.9
    kI: float = 0.7
    kP: float = 0.4
    dt_min: float = 1e-12
    dt_max: float = 1.0
    max_factor: float = 5.0
    min_factor: float = 0.2
    atol: float = 1e-6
    rtol: float = 1e-4


@dataclass
class Model:
    """Stand-in for MOLModel (moljax/core/model.py:34-118): BC kinds + reaction."""
    grid: object
    bc_kinds: Dict[str, int]
    params: Dict[str, float]
    reaction: Callable | None = None

    def apply_bcs(self, y):
        return mol.apply_bc(y, self.grid, self.bc_kinds)

    def nonlinear_rhs(self, y):
        return self.reaction(y)


def gray_scott_periodic(grid, Du, Dv, F, k):
    """moljax/core/model.py:213-292 + 529-584 -> (model, lam, diffusivities)."""
    model = Model(grid, {"u": mol.PERIODIC, "v": mol.PERIODIC},
                  {"Du": Du, "Dv": Dv, "F": F, "k": k},
                  lambda y: mol.gray_scott_reaction(y, F, k))
    lam = mol.fd_symbol_2d(grid.ny, grid.nx, grid.dy, grid.dx)
    return model, lam, {"u": Du, "v": Dv}


def _axpy(y, a, x):
    return {kk: y[kk] + a * x[kk] for kk in y}


def imex_euler_step(model, y, dt, lam, diff):
    """moljax/core/stepping.py:317-367."""
    y = model.apply_bcs(y)
    N = model.nonlinear_rhs(y) if model.reaction else {k: np.zeros_like(f) for k, f in y.items()}
    y_new = mol.apply_diffusion_inverse_fft(_axpy(y, dt, N), model.grid, dt, diff, lam)
    return model.apply_bcs(y_new)


def imex_ssprk2_step(model, y, dt, lam, diff):
    """moljax/core/stepping.py:438-495: y1 = H(dt)(y + dt N(y)); y2 = H(dt)(y1 + dt N(y1));
    y_new = (y + y2)/2, BCs applied after each stage."""
    y = model.apply_bcs(y)

    def N(z):
        return model.nonlinear_rhs(z) if model.reaction else {k: np.zeros_like(f) for k, f in z.items()}
    y1 = model.apply_bcs(mol.apply_diffusion_inverse_fft(_axpy(y, dt, N(y)), model.grid, dt, diff, lam))
    y2 = model.apply_bcs(mol.apply_diffusion_inverse_fft(_axpy(y1, dt, N(y1)), model.grid, dt, diff, lam))
    return model.apply_bcs({k: 0.5 * y[k] + 0.5 * y2[k] for k in y})


def imex_strang_step(model, y, dt, lam, diff):
    """moljax/core/stepping.py:370-435: H(dt/2) -> Heun reaction(dt) -> H(dt/2)."""
    h = dt / 2.0
    y = model.apply_bcs(y)
    ys = mol.apply_diffusion_inverse_fft(y, model.grid, h, diff, lam)
    ys = model.apply_bcs(ys)
    if model.reaction is not None:
        R1 = model.nonlinear_rhs(ys)
        yt = model.apply_bcs(_axpy(ys, dt, R1))
        R2 = model.nonlinear_rhs(yt)
        yd = _axpy(ys, 0.5 * dt, {k: R1[k] + R2[k] for k in R1})
    else:
        yd = ys
    yd = model.apply_bcs(yd)
    y_new = mol.apply_diffusion_inverse_fft(yd, model.grid, h, diff, lam)
    return model.apply_bcs(y_new)


def estimate_error_imex_doubling(model, y, dt, lam, diff, use_strang=True):
    """moljax/core/stepping.py:566-608: returns (y_half2, y_half2 - y_full)."""
    step = imex_strang_step if use_strang else imex_euler_step
    y_full = step(model, y, dt, lam, diff)
    y_h1 = step(model, y, dt / 2.0, lam, diff)
    y_h2 = step(model, y_h1, dt / 2.0, lam, diff)
    return y_h2, {k: y_h2[k] - y_full[k] for k in y_h2}


def imex_cfl_dt(grid, params, cfl):
    """moljax/core/dt_policy.py:430-502 (advection, wave, reaction 0.5/(F+k); no diffusion)."""
    dx = grid.min_dx if hasattr(grid, "min_dx") else grid.dx
    dt = cfl.dt_max
    v = abs(params.get("vx", 0.0)) + abs(params.get("vy", 0.0))
    dt = min(dt, cfl.cfl_advection * dx / v if v > 1e-14 else cfl.dt_max)
    K, rho = params.get("K", 0.0), params.get("rho", 1.0)
    c = max(params.get("wave_speed", 0.0), math.sqrt(K / rho) if K > 1e-14 else 0.0)
    dt = min(dt, cfl.cfl_wave * dx / c if c > 1e-14 else cfl.dt_max)
    rate = max(params.get("F", 0.0) + params.get("k", 0.0), params.get("r", 0.0))
    dt = min(dt, 0.5 / rate if rate > 1e-14 else cfl.dt_max)
    return float(np.clip(cfl.safety * dt, cfl.dt_min, cfl.dt_max))


def pid_controller_dt(dt_old, err, prev_err, pid, order):
    """moljax/core/dt_policy.py:178-227 -> (dt_new, new prev_err)."""
    kI, kP = pid.kI / order, pid.kP / order
    e = max(err, 1e-10)
    pe = max(prev_err, 1e-10)
    fac = (1.0 / e) ** kI * (pe / e) ** kP
    fac = min(max(fac * pid.safety, pid.min_factor), pid.max_factor)
    return min(max(dt_old * fac, pid.dt_min), pid.dt_max), err


def handle_rejected_step(dt_old, err, pid, order):
    """moljax/core/dt_policy.py:230-268."""
    kI = pid.kI / order
    fac = pid.safety * (1.0 / max(err, 1.0)) ** kI
    fac = min(max(fac, pid.min_factor), 1.0)
    return min(max(dt_old * fac, pid.dt_min), pid.dt_max)


def propose_dt_imex(grid, params, dt_old, err, prev_err, cfl, pid, order):
    """moljax/core/dt_policy.py:544-610 -> (dt_new, prev_err_after)."""
    if err <= 1.0:
        dt_a, pe = pid_controller_dt(dt_old, err, prev_err, pid, order)
    else:
        dt_a, pe = handle_rejected_step(dt_old, err, pid, order), prev_err
    dt_f = min(dt_a, imex_cfl_dt(grid, params, cfl))
    return min(max(dt_f, pid.dt_min), pid.dt_max), pe


@dataclass
class AdaptiveResult:
    """moljax/core/stepping.py:710-720."""
    t_final: float
    y_final: dict
    t_history: np.ndarray
    y_history: dict
    dt_history: np.ndarray
    n_steps: int
    n_accepted: int
    n_rejected: int
    status: int
    err_history: list = field(default_factory=list)


def adaptive_integrate_imex(model, y0, t0, t_end, dt0, lam, diff, use_strang=True,
                            max_steps=10000, cfl=None, pid=None, save_every=1,
                            keep_history=True, max_attempts=None):
    """moljax/core/stepping.py:1146-1371 (the accept/reject state machine).

    ``keep_history=False`` skips the y history copies (t/dt histories kept).
    ``max_attempts`` bounds the loop for CPU sampling (None = unbounded, as the
    reference); ``err_history`` records (t, dt_clamped, err_ratio, accepted).
    """
    cfl = cfl or CFLParams()
    pid = pid or PIDParams()
    order = 2 if use_strang else 1
    grid = model.grid
    dt = min(float(dt0), imex_cfl_dt(grid, model.params, cfl))
    max_saves = max_steps // save_every + 1
    t_hist = np.zeros(max_saves)
    dt_hist = np.zeros(max_saves)
    y_hist = {k: [] for k in y0} if keep_history else None
    t_hist[0] = t0
    if keep_history:
        for k in y0:
            y_hist[k].append(mol.interior(y0[k], grid).copy())
    t, y = float(t0), y0
    prev_err = 1.0
    write_idx, n_acc, n_rej, status = 1, 0, 0, RUNNING
    errs = []
    attempts = 0
    while status == RUNNING and t < t_end and write_idx < max_saves:
        if max_attempts is not None and attempts >= max_attempts:
            break
        attempts += 1
        dtc = min(dt, t_end - t)
        y_new, err = estimate_error_imex_doubling(model, y, dtc, lam, diff, use_strang)
        e = max(mol.scaled_error_norm(err, y_new, grid, pid.atol, pid.rtol), 1e-10)
        finite = mol.is_finite(y_new)
        accept = (e <= 1.0) and finite
        dt_new, pe_new = propose_dt_imex(grid, model.params, dtc, e, prev_err, cfl, pid, order)
        errs.append((t, dtc, e, accept))
        if accept:
            if n_acc % save_every == 0:
                t_hist[write_idx] = t + dtc
                if keep_history:
                    for k in y_new:
                        y_hist[k].append(mol.interior(y_new[k], grid).copy())
                dt_hist[write_idx - 1] = dtc
                write_idx += 1
            t = t + dtc
            y = y_new
            dt = dt_new
            prev_err = pe_new
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
    if keep_history:
        y_hist = {k: np.array(v) for k, v in y_hist.items()}
    return AdaptiveResult(t, y, t_hist, y_hist, dt_hist, write_idx, n_acc, n_rej, status, errs)


def integrate_imex_fixed_dt(model, y0, t0, t_end, dt, lam, diff, use_strang=True):
    """moljax/core/stepping.py:1374-1436: n_steps = int((t_end-t0)/dt)+1 fixed steps."""
    n = int((t_end - t0) / dt) + 1
    step = imex_strang_step if use_strang else imex_euler_step
    y = y0
    ts, ys = [], []
    t = t0
    for _ in range(n):
        y = step(model, y, dt, lam, diff)
        t = t + dt
        ts.append(t)
        ys.append(y)
    return np.array(ts), ys, y
