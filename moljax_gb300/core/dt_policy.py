"""Time-step policy parameters and host-side controller formulas.

``CFLParams``/``PIDParams``/``ControllerState`` and the scalar formulas
mirror moljax/core/dt_policy.py:28-610.  Inside the adaptive drivers the same
formulas run on the GPU (controller kernel in ``csrc/imex.cu``); the host
versions here serve the initial step size and direct callers.

README spellings are accepted as aliases (README.md:132-138):
``CFLParams(cfl_target=, safety_factor=)`` -> ``cfl_advection``/``safety``;
``PIDParams(ki=, kp=, kd=)`` -> ``kI``/``kP``; ``kd`` is accepted and ignored
(the reference controller is PI only).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import NamedTuple, Optional


@dataclass(frozen=True, init=False)
class CFLParams:
    safety: float
    dt_min: float
    dt_max: float
    cfl_advection: float
    cfl_diffusion: float
    cfl_wave: float

    def __init__(self, safety: float = 0.9, dt_min: float = 1e-12, dt_max: float = 1.0,
                 cfl_advection: float = 0.5, cfl_diffusion: float = 0.25, cfl_wave: float = 0.5,
                 *, cfl_target: Optional[float] = None, safety_factor: Optional[float] = None):
        if safety_factor is not None:
            safety = safety_factor
        if cfl_target is not None:
            cfl_advection = cfl_target
        for k, v in dict(safety=safety, dt_min=dt_min, dt_max=dt_max, cfl_advection=cfl_advection,
                         cfl_diffusion=cfl_diffusion, cfl_wave=cfl_wave).items():
            object.__setattr__(self, k, float(v))


@dataclass(frozen=True, init=False)
class PIDParams:
    safety: float
    kI: float
    kP: float
    dt_min: float
    dt_max: float
    max_factor: float
    min_factor: float
    atol: float
    rtol: float

    def __init__(self, safety: float = 0.9, kI: float = 0.7, kP: float = 0.4,
                 dt_min: float = 1e-12, dt_max: float = 1.0, max_factor: float = 5.0,
                 min_factor: float = 0.2, atol: float = 1e-6, rtol: float = 1e-4, *,
                 ki: Optional[float] = None, kp: Optional[float] = None,
                 kd: Optional[float] = None):
        if ki is not None:
            kI = ki
        if kp is not None:
            kP = kp
        del kd  # PI controller only (moljax/core/dt_policy.py:178-227)
        for k, v in dict(safety=safety, kI=kI, kP=kP, dt_min=dt_min, dt_max=dt_max,
                         max_factor=max_factor, min_factor=min_factor, atol=atol,
                         rtol=rtol).items():
            object.__setattr__(self, k, float(v))


class ControllerState(NamedTuple):
    """moljax/core/dt_policy.py:81-101."""
    prev_err_ratio: float
    prevprev_err_ratio: float
    consecutive_rejects: int


def create_initial_controller_state(dtype=None) -> ControllerState:
    return ControllerState(1.0, 1.0, 0)


def _clip(x, lo, hi):
    if math.isnan(x):
        return x
    return min(max(x, lo), hi)


def pid_controller_dt(dt_old, err_ratio, controller_state: ControllerState,
                      pid_params: PIDParams, order: int = 4):
    """moljax/core/dt_policy.py:178-227."""
    kI = pid_params.kI / order
    kP = pid_params.kP / order
    e = max(err_ratio, 1e-10)
    pe = max(controller_state.prev_err_ratio, 1e-10)
    fac = (1.0 / e) ** kI * (pe / e) ** kP
    fac = _clip(fac * pid_params.safety, pid_params.min_factor, pid_params.max_factor)
    dt_new = _clip(dt_old * fac, pid_params.dt_min, pid_params.dt_max)
    return dt_new, ControllerState(err_ratio, controller_state.prev_err_ratio, 0)


def handle_rejected_step(dt_old, err_ratio, controller_state: ControllerState,
                         pid_params: PIDParams, order: int = 4):
    """moljax/core/dt_policy.py:230-268."""
    kI = pid_params.kI / order
    fac = pid_params.safety * (1.0 / max(err_ratio, 1.0)) ** kI
    fac = _clip(fac, pid_params.min_factor, 1.0)
    dt_new = _clip(dt_old * fac, pid_params.dt_min, pid_params.dt_max)
    return dt_new, ControllerState(controller_state.prev_err_ratio,
                                   controller_state.prevprev_err_ratio,
                                   controller_state.consecutive_rejects + 1)


def compute_error_order(method: int) -> int:
    """moljax/core/dt_policy.py:411-423."""
    orders = [1, 3, 4, 1, 2, 2, 1, 2]
    return orders[min(int(method), len(orders) - 1)]


def _params_get(params, key, default=0.0):
    v = params.get(key, default)
    return float(v) if not isinstance(v, type) else default


def heisenberg_cfl_dt(grid, params, cfl_params: CFLParams) -> float:
    """moljax/core/dt_policy.py:104-175 (advection, diffusion, wave limits)."""
    dx, dx2 = grid.min_dx, grid.min_dx2
    dt = cfl_params.dt_max
    v = abs(_params_get(params, "vx")) + abs(_params_get(params, "vy"))
    dt = min(dt, cfl_params.cfl_advection * dx / v if v > 1e-14 else cfl_params.dt_max)
    Dm = max(_params_get(params, "D"), _params_get(params, "Du"), _params_get(params, "Dv"))
    dt = min(dt, cfl_params.cfl_diffusion * dx2 / Dm if Dm > 1e-14 else cfl_params.dt_max)
    K, rho = _params_get(params, "K"), _params_get(params, "rho", 1.0)
    c = max(_params_get(params, "wave_speed"), math.sqrt(K / rho) if K > 1e-14 else 0.0)
    dt = min(dt, cfl_params.cfl_wave * dx / c if c > 1e-14 else cfl_params.dt_max)
    return _clip(cfl_params.safety * dt, cfl_params.dt_min, cfl_params.dt_max)


def imex_cfl_dt(grid, params, cfl_params: CFLParams) -> float:
    """moljax/core/dt_policy.py:430-502 (no diffusion limit; reaction 0.5/(F+k))."""
    dx = grid.min_dx
    dt = cfl_params.dt_max
    v = abs(_params_get(params, "vx")) + abs(_params_get(params, "vy"))
    dt = min(dt, cfl_params.cfl_advection * dx / v if v > 1e-14 else cfl_params.dt_max)
    K, rho = _params_get(params, "K"), _params_get(params, "rho", 1.0)
    c = max(_params_get(params, "wave_speed"), math.sqrt(K / rho) if K > 1e-14 else 0.0)
    dt = min(dt, cfl_params.cfl_wave * dx / c if c > 1e-14 else cfl_params.dt_max)
    rate = max(_params_get(params, "F") + _params_get(params, "k"), _params_get(params, "r"))
    dt = min(dt, 0.5 / rate if rate > 1e-14 else cfl_params.dt_max)
    return _clip(cfl_params.safety * dt, cfl_params.dt_min, cfl_params.dt_max)


def propose_dt_imex(grid, params, state, t, dt_old, err_ratio, controller_state,
                    cfl_params: Optional[CFLParams] = None, pid_params: Optional[PIDParams] = None,
                    order: int = 2):
    """moljax/core/dt_policy.py:544-610 (host form of the device controller)."""
    cfl_params = cfl_params or CFLParams()
    pid_params = pid_params or PIDParams()
    if err_ratio <= 1.0:
        dt_a, st = pid_controller_dt(dt_old, err_ratio, controller_state, pid_params, order)
    else:
        dt_a, st = handle_rejected_step(dt_old, err_ratio, controller_state, pid_params, order)
    dt_f = min(dt_a, imex_cfl_dt(grid, params, cfl_params))
    return _clip(dt_f, pid_params.dt_min, pid_params.dt_max), st


def implicit_robustness_dt(dt_old, nk_stats, dt_min: float = 1e-12, dt_max: float = 1.0,
                           growth_factor: float = 1.2, shrink_factor: float = 0.5,
                           fast_iters_threshold: int = 3) -> float:
    """moljax/core/dt_policy.py:279-321: halve on Newton failure, grow 1.2x when Newton
    converged within fast_iters_threshold iterations, clip to [dt_min, dt_max]."""
    dt = dt_old if nk_stats.converged else dt_old * shrink_factor
    if nk_stats.converged and nk_stats.newton_iters <= fast_iters_threshold:
        dt = min(dt * growth_factor, dt_max)
    return _clip(dt, dt_min, dt_max)


def propose_dt(method: int, grid, params, state, t, dt_old, err_ratio,
               controller_state: ControllerState, nk_stats=None,
               cfl_params: Optional[CFLParams] = None, pid_params: Optional[PIDParams] = None,
               order: int = 4):
    """moljax/core/dt_policy.py:324-408: PI (accepted) or reject formula, the CFL limit for
    explicit methods, implicit_robustness_dt for implicit ones, final clamp.
    Returns (dt, new ControllerState).  The native drivers run the same rule on the device
    (explicit) or in their C++ loop (implicit)."""
    cfl_params = cfl_params or CFLParams()
    pid_params = pid_params or PIDParams()
    if err_ratio <= 1.0:
        dt_a, st = pid_controller_dt(dt_old, err_ratio, controller_state, pid_params, order)
    else:
        dt_a, st = handle_rejected_step(dt_old, err_ratio, controller_state, pid_params, order)
    if method < 3:
        dt_a = min(dt_a, heisenberg_cfl_dt(grid, params, cfl_params))
    if nk_stats is not None and method >= 3:
        dt_a = implicit_robustness_dt(dt_a, nk_stats)
    return _clip(dt_a, pid_params.dt_min, pid_params.dt_max), st


def estimate_reaction_stiffness(state, params) -> float:
    """Reaction stiffness bound (dt_policy.py:505-541): Gray-Scott max(F + k, v^2 + F,
    2 u v + F + k) from the state's maxima; Fisher-KPP r."""
    s = 0.0
    if "F" in params and "k" in params:
        F, k = float(params["F"]), float(params["k"])
        s = max(s, F + k)
        if "u" in state and "v" in state:
            vm = float(state["v"].abs().max())
            um = float(state["u"].abs().max())
            s = max(s, vm ** 2 + F, 2 * um * vm + F + k)
    if "r" in params:
        s = max(s, float(params["r"]))
    return s
