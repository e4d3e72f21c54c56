"""Time integration drivers (moljax/core/stepping.py drop-in, GPU-native).

IMEX paths run in the native library: one IMEX-Strang step
(``mjx_imex_strang_step2d``) and the whole adaptive loop
(``mjx_imex_adaptive2d``), where step doubling, the scaled error norm, the PI
controller and the accept/reject bookkeeping stay on the device inside a CUDA
graph with a conditional while node -- the counterpart of the reference's
``lax.while_loop`` (stepping.py:1225-1348) with no host synchronisation per
step.

``adaptive_integrate`` accepts the reference signature
(model, y0, t0, t_end, dt0, method, ...) and the README form
(model, t_span=, integrator=, rtol=, atol=).
"""

from __future__ import annotations

import ctypes as C
from enum import IntEnum
from typing import Dict, NamedTuple, Optional

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core import stencil
from moljax_gb300.core.dt_policy import CFLParams, PIDParams, imex_cfl_dt
from moljax_gb300.core.fft_solvers import _plan_of, create_fft_cache, workspace


class IntegratorType(IntEnum):
    """moljax/core/stepping.py:48-57, plus ETDRK4 (an IntegratorType in the README)."""
    EULER = 0
    SSPRK3 = 1
    RK4 = 2
    BE = 3
    CN = 4
    BDF2 = 5
    IMEX_EULER = 6
    IMEX_STRANG = 7
    ETDRK4 = 8


class AdaptiveResult(NamedTuple):
    """moljax/core/stepping.py:710-720."""
    t_final: float
    y_final: Dict[str, torch.Tensor]
    t_history: torch.Tensor
    y_history: Optional[Dict[str, torch.Tensor]]
    dt_history: torch.Tensor
    n_steps: int
    n_accepted: int
    n_rejected: int
    status: int


def _problem(model, diffusivities, cfl_params, max_attempts=0):
    names = model.field_names
    if len(names) > 4:
        raise NotImplementedError("at most 4 fields per native IMEX call")
    rx = model.reaction_kind
    p = N.ImexProblemC()
    p.reaction = rx
    p.nfields = len(names)
    for i, n in enumerate(names):
        p.D[i] = float(diffusivities.get(n, 0.0))
    p.F = float(model.params.get("F", 0.0))
    p.k = float(model.params.get("k", 0.0))
    p.r = float(model.params.get("r", 0.0))
    p.dt_cfl = imex_cfl_dt(model.grid, model.params, cfl_params)
    p.use_strang = 1
    p.max_attempts = int(max_attempts)
    return p


def _periodic_only(model):
    from moljax_gb300.core.bc import BCType
    for n, s in model.bc_spec.items():
        if s.kind != BCType.PERIODIC:
            raise NotImplementedError("FFT IMEX paths need periodic BCs (as the reference)")


def imex_strang_step(model, y, t, dt, fft_cache, diffusivities):
    """One IMEX-Strang step H(dt/2) R(dt) H(dt/2) (moljax/core/stepping.py:370-435)."""
    _periodic_only(model)
    grid = model.grid
    names = model.field_names
    interior = stencil.unpad(stencil.stack(y, names), grid)
    plan = _plan_of(fft_cache, grid.ny, grid.nx, interior.dtype)
    prob = _problem(model, diffusivities, CFLParams())
    lib = N.lib()
    ws = workspace(lib.mjx_imex2d_ws_bytes(grid.ny, grid.nx, len(names), plan.code), plan.device,
                   "imex")
    out = torch.empty_like(interior)
    N.check("mjx_imex_strang_step2d", lib.mjx_imex_strang_step2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, C.byref(prob), float(dt),
        N.ptr(interior), N.ptr(out), N.ptr(ws), ws.numel(), N.stream_ptr(plan.device)))
    padded = stencil.pad_interior(out, grid, model.bc_spec, names, t + dt, model.params)
    return {n: padded[i] for i, n in enumerate(names)}


def integrate_imex_fixed_dt(model, y0, t0, t_end, dt, fft_cache, diffusivities,
                            use_strang: bool = True, save_every: int = 1):
    """moljax/core/stepping.py:1374-1436: int((t_end-t0)/dt)+1 fixed steps."""
    if not use_strang:
        raise NotImplementedError("IMEX-Euler fixed-dt path is not built")
    n = int((t_end - t0) / dt) + 1
    y = y0
    t = t0
    ts, ys = [], []
    for _ in range(n):
        y = imex_strang_step(model, y, t, dt, fft_cache, diffusivities)
        t = t + dt
        ts.append(t)
        ys.append({k: stencil.unpad(v[None], model.grid)[0] for k, v in y.items()})
    t_out = torch.tensor(ts, dtype=torch.float64)
    y_out = {k: torch.stack([s[k] for s in ys]) for k in y0}
    return t_out, y_out, y


def adaptive_integrate_imex(model, y0, t0, t_end, dt0, fft_cache=None, diffusivities=None,
                            use_strang: bool = True, max_steps: int = 10000,
                            cfl_params: Optional[CFLParams] = None,
                            pid_params: Optional[PIDParams] = None, save_every: int = 1,
                            save_y_history: bool = True, max_attempts: int = 0,
                            precision: Optional[str] = None) -> AdaptiveResult:
    """Adaptive IMEX with step doubling and PI control (stepping.py:1146-1371).

    Runs entirely on the GPU as one graph launch.  ``save_y_history=False``
    skips the (max_steps//save_every+1) x state history buffer; t/dt histories
    are always kept.  ``max_attempts`` caps accepted+rejected attempts
    (default 20*max_steps+1000) so the device loop always terminates.

    ``precision``: ``"fp64"`` (FP64 everywhere; default for float64 models),
    ``"fp32"`` (FP32 state and transforms) or ``"mixed"`` (float-float spectral state,
    FP32 transforms of the reaction increments; FP32 in/out; no y history).
    float32 models default to ``"fp32"``.
    """
    if not use_strang:
        raise NotImplementedError("adaptive IMEX-Euler is not built; use_strang=True")
    _periodic_only(model)
    cfl_params = cfl_params or CFLParams()
    pid_params = pid_params or PIDParams()
    grid = model.grid
    names = model.field_names
    if diffusivities is None:
        diffusivities = model.diffusivities()
    if fft_cache is None:
        fft_cache = model.metadata.get("fft_cache") or create_fft_cache(grid, model.dtype)
    interior = stencil.unpad(stencil.stack(y0, names), grid)
    plan = _plan_of(fft_cache, grid.ny, grid.nx, interior.dtype)
    prob = _problem(model, diffusivities, cfl_params, max_attempts)
    if precision is None:
        precision = "fp64" if interior.dtype == torch.float64 else "fp32"
    if precision == "mixed":
        return _adaptive_mixed(model, interior, plan, prob, pid_params, t0, t_end, dt0, max_steps,
                               save_every)
    if precision not in ("fp32", "fp64"):
        raise ValueError(f"precision must be 'fp32', 'fp64' or 'mixed', not {precision!r}")
    if (precision == "fp64") != (interior.dtype == torch.float64):
        raise TypeError(f"precision {precision!r} needs a {'float64' if precision == 'fp64' else 'float32'} state")
    pid = N.PIDParamsC(pid_params.safety, pid_params.kI, pid_params.kP, pid_params.dt_min,
                       pid_params.dt_max, pid_params.max_factor, pid_params.min_factor,
                       pid_params.atol, pid_params.rtol)
    lib = N.lib()
    dev = plan.device
    max_saves = max_steps // save_every + 1
    ws = workspace(lib.mjx_imex2d_ws_bytes(grid.ny, grid.nx, len(names), plan.code), dev, "imex")
    y_final = torch.empty_like(interior)
    t_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    dt_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    y_hist = (torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype, device=dev)
              if save_y_history else None)
    res = N.AdaptiveResultC()
    N.check("mjx_imex_adaptive2d", lib.mjx_imex_adaptive2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, C.byref(prob), C.byref(pid),
        float(t0), float(t_end), float(dt0), int(max_steps), int(save_every), N.ptr(interior),
        N.ptr(y_final), C.cast(C.c_void_p(t_hist.data_ptr()), C.POINTER(C.c_double)),
        C.cast(C.c_void_p(dt_hist.data_ptr()), C.POINTER(C.c_double)), N.ptr(y_hist),
        N.ptr(ws), ws.numel(), C.byref(res), N.stream_ptr(dev)))
    padded = stencil.pad_interior(y_final, grid, model.bc_spec, names, res.t_final, model.params)
    y_fin = {n: padded[i] for i, n in enumerate(names)}
    y_history = ({n: y_hist[:, i] for i, n in enumerate(names)} if y_hist is not None else None)
    return AdaptiveResult(res.t_final, y_fin, t_hist, y_history, dt_hist, res.n_saved,
                          res.n_accepted, res.n_rejected, res.status)


def _adaptive_mixed(model, interior, plan, prob, pid_params, t0, t_end, dt0, max_steps,
                    save_every) -> AdaptiveResult:
    from moljax_gb300.core.fft_solvers import get_plan
    grid = model.grid
    names = model.field_names
    p32 = get_plan(plan.ny, plan.nx, plan.dy, plan.dx, plan.symbol, torch.float32, plan.device)
    p64 = get_plan(plan.ny, plan.nx, plan.dy, plan.dx, plan.symbol, torch.float64, plan.device)
    pid = N.PIDParamsC(pid_params.safety, pid_params.kI, pid_params.kP, pid_params.dt_min,
                       pid_params.dt_max, pid_params.max_factor, pid_params.min_factor,
                       pid_params.atol, pid_params.rtol)
    lib = N.lib()
    dev = plan.device
    max_saves = max_steps // save_every + 1
    ws = workspace(lib.mjx_imex2d_mixed_ws_bytes(grid.ny, grid.nx, len(names)), dev, "imex_mixed")
    y_final = torch.empty_like(interior)
    t_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    dt_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    res = N.AdaptiveResultC()
    N.check("mjx_imex_adaptive2d_mixed", lib.mjx_imex_adaptive2d_mixed(
        N.ptr(p32.buf), N.ptr(p64.buf), C.byref(p32.cgrid), N.dtype_code(interior.dtype),
        C.byref(prob), C.byref(pid), float(t0), float(t_end), float(dt0), int(max_steps),
        int(save_every), N.ptr(interior), N.ptr(y_final),
        C.cast(C.c_void_p(t_hist.data_ptr()), C.POINTER(C.c_double)),
        C.cast(C.c_void_p(dt_hist.data_ptr()), C.POINTER(C.c_double)),
        N.ptr(ws), ws.numel(), C.byref(res), N.stream_ptr(dev)))
    padded = stencil.pad_interior(y_final, grid, model.bc_spec, names, res.t_final, model.params)
    y_fin = {n: padded[i] for i, n in enumerate(names)}
    return AdaptiveResult(res.t_final, y_fin, t_hist, None, dt_hist, res.n_saved, res.n_accepted,
                          res.n_rejected, res.status)


def adaptive_integrate(model, y0=None, t0: float = 0.0, t_end: Optional[float] = None,
                       dt0: float = 1.0, method: int = IntegratorType.RK4, max_steps: int = 10000,
                       cfl_params: Optional[CFLParams] = None,
                       pid_params: Optional[PIDParams] = None, preconditioner=None,
                       nk_params=None, save_every: int = 1, *, t_span=None, integrator=None,
                       rtol: Optional[float] = None, atol: Optional[float] = None, **kw):
    """Reference form (stepping.py:723-1021) or README form (README.md:75-80).

    IMEX_STRANG routes to ``adaptive_integrate_imex`` (the reference's real
    IMEX driver).  Other methods are dispatched to their native drivers as they
    are built; unbuilt ones raise NotImplementedError.
    """
    if t_span is not None:
        t0, t_end = float(t_span[0]), float(t_span[1])
    if integrator is not None:
        method = integrator
    if t_end is None:
        raise TypeError("adaptive_integrate needs t_end (or t_span=)")
    if rtol is not None or atol is not None:
        base = pid_params or PIDParams()
        pid_params = PIDParams(base.safety, base.kI, base.kP, base.dt_min, base.dt_max,
                               base.max_factor, base.min_factor,
                               base.atol if atol is None else atol,
                               base.rtol if rtol is None else rtol)
    if y0 is None:
        y0 = kw.pop("initial_state", None)
        if y0 is None:
            raise TypeError("adaptive_integrate needs an initial state y0")
    method = IntegratorType(int(method))
    if method == IntegratorType.ETDRK4:
        # the reference has no adaptive ETDRK4: fixed steps of dt0 over the span
        from moljax_gb300.core.fft_integrators import etd_integrate
        y, tf = etd_integrate(model, y0, t0, t_end, dt0, kw.pop("symbol", "fd"))
        n = int(round((tf - t0) / dt0))
        return AdaptiveResult(tf, y, torch.tensor([t0, tf], dtype=torch.float64), None,
                              torch.tensor([dt0], dtype=torch.float64), 2, n, 0, 0)
    if method == IntegratorType.IMEX_STRANG:
        return adaptive_integrate_imex(model, y0, t0, t_end, dt0, None, None, True, max_steps,
                                       cfl_params, pid_params, save_every, **kw)
    raise NotImplementedError(f"{method.name} adaptive driver is not built on the GPU path")
