"""Time integration drivers (moljax/core/stepping.py drop-in, GPU-native).

IMEX paths run in the native library: one IMEX-Strang or IMEX-Euler step
(``mjx_imex_strang_step2d``) and the whole adaptive loop
(``mjx_imex_adaptive2d``), where step doubling, the scaled error norm, the PI
controller and the accept/reject bookkeeping stay on the device inside a CUDA
graph with a conditional while node -- the counterpart of the reference's
``lax.while_loop`` (stepping.py:1225-1348) with no host synchronisation per
step.

``adaptive_integrate`` accepts the reference signature
(model, y0, t0, t_end, dt0, method, ...) and the README form
(model, t_span=, integrator=, rtol=, atol=).  EULER/SSPRK3/RK4 (``euler_step``,
``ssprk3_step``, ``rk4_step``, fixed and adaptive) run fused stencil-stage kernels
for the built-in reaction-advection-diffusion models with any ghost BCs.  BE/CN/BDF2 (``be_step``,
``cn_step``, ``bdf2_step``, ``integrate_fixed_dt``, ``adaptive_integrate``) run
on the native Newton-Krylov solver for the variable-diffusion model.
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


def _problem(model, diffusivities, cfl_params, max_attempts=0, use_strang=True):
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
    p.use_strang = 1 if use_strang else 0
    p.max_attempts = int(max_attempts)
    return p


def _pid_c(pid_params):
    """PIDParams -> the C struct (moljax/core/dt_policy.py:49-78 fields)."""
    return N.PIDParamsC(pid_params.safety, pid_params.kI, pid_params.kP, pid_params.dt_min,
                        pid_params.dt_max, pid_params.max_factor, pid_params.min_factor,
                        pid_params.atol, pid_params.rtol)


def _periodic_only(model):
    from moljax_gb300.core.bc import BCType
    for n, s in model.bc_spec.items():
        if s.kind != BCType.PERIODIC:
            raise NotImplementedError("FFT IMEX paths need periodic BCs (as the reference)")


def imex_strang_step(model, y, t, dt, fft_cache, diffusivities):
    """One IMEX-Strang step H(dt/2) R(dt) H(dt/2) (moljax/core/stepping.py:370-435)."""
    return _imex_step(model, y, t, dt, fft_cache, diffusivities, True)


def imex_euler_step(model, y, t, dt, fft_cache, diffusivities):
    """One IMEX-Euler step H(dt) (y + dt N(y)) (moljax/core/stepping.py:317-367)."""
    return _imex_step(model, y, t, dt, fft_cache, diffusivities, False)


# ------------------------------------------------------------------ grids of any size
def _reaction_args(model):
    rx = model.reaction_kind
    p = model.params
    return rx, float(p.get("F", 0.0)), float(p.get("k", 0.0)), float(p.get("r", 1.0))


def _imex_interior_general(model, plan, interior, dt, diffusivities, use_strang):
    """One IMEX step on interiors (nf, ny, nx) of a grid of any size: the general spectral
    plan for H, the native Heun / Euler reaction kernels for R (the reaction is pointwise and
    H acts on interiors, so the intermediate ghost fills of the reference change nothing)."""
    names = model.field_names
    D = [float(diffusivities.get(n, 0.0)) for n in names]
    diffusive = [i for i, d in enumerate(D) if d > 1e-14]

    def H(x, h):
        out = x.clone()
        if diffusive:
            sel = torch.tensor(diffusive, device=x.device)
            out[sel] = plan.apply(x[sel].contiguous(), [D[i] for i in diffusive], h, N.MULT_HELMHOLTZ)
        return out

    rx, F, k, r = _reaction_args(model)
    nf = interior.shape[0]
    npts = interior[0].numel()

    def react(x, h, euler):
        out = torch.empty_like(x)
        N.check("mjx_reaction_step2d", N.lib().mjx_reaction_step2d(
            N.ptr(x), N.ptr(out), nf, npts, rx, F, k, r, float(h), int(euler), N.dtype_code(x.dtype),
            N.stream_ptr(x.device)))
        return out

    if use_strang:  # H(dt/2) R_heun(dt) H(dt/2)
        return H(react(H(interior, 0.5 * dt), dt, 0), 0.5 * dt)
    return H(react(interior, dt, 1), dt)  # H(dt) (y + dt N(y))


def _imex_step(model, y, t, dt, fft_cache, diffusivities, use_strang):
    _periodic_only(model)
    grid = model.grid
    names = model.field_names
    interior = stencil.unpad(stencil.stack(y, names), grid)
    plan = _plan_of(fft_cache, grid.ny, grid.nx, interior.dtype)
    if getattr(plan, "general", False):
        out = _imex_interior_general(model, plan, interior, dt, diffusivities, use_strang)
        padded = stencil.pad_interior(out, grid, model.bc_spec, names, t + dt, model.params)
        return {n: padded[i] for i, n in enumerate(names)}
    prob = _problem(model, diffusivities, CFLParams(), use_strang=use_strang)
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
    n = int((t_end - t0) / dt) + 1
    y = y0
    t = t0
    ts, ys = [], []
    for _ in range(n):
        y = _imex_step(model, y, t, dt, fft_cache, diffusivities, use_strang)
        t = t + dt
        ts.append(t)
        ys.append(y)
    t_out = torch.tensor(ts, dtype=torch.float64)
    y_out = {k: torch.stack([s[k] for s in ys]) for k in y0}  # padded, as the scan outputs
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
    ``save_y_history="host"`` streams the saved states into pinned host memory as
    the loop runs (the history never occupies HBM; O(max_saves * n) histories at
    1024^2 stay on the host side of NVLink-C2C).

    ``use_strang=False`` runs IMEX-Euler under the same step doubling with
    error order 1 (stepping.py:1193); it has the "fp32" and "fp64" forms.
    """
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
    if getattr(plan, "general", False):
        if precision == "mixed":
            raise NotImplementedError("the mixed-precision form needs a power-of-two grid")
        return _adaptive_imex_general(model, interior, plan, diffusivities, use_strang, t0, t_end, dt0,
                                      max_steps, cfl_params, pid_params, save_every, save_y_history,
                                      max_attempts)
    prob = _problem(model, diffusivities, cfl_params, max_attempts, use_strang)
    if precision is None:
        precision = "fp64" if interior.dtype == torch.float64 else "fp32"
    if precision == "mixed":
        if not use_strang:
            raise NotImplementedError("the mixed-precision form is built for IMEX-Strang only")
        return _adaptive_mixed(model, interior, plan, prob, pid_params, t0, t_end, dt0, max_steps,
                               save_every)
    if precision not in ("fp32", "fp64"):
        raise ValueError(f"precision must be 'fp32', 'fp64' or 'mixed', not {precision!r}")
    if (precision == "fp64") != (interior.dtype == torch.float64):
        raise TypeError(f"precision {precision!r} needs a {'float64' if precision == 'fp64' else 'float32'} state")
    pid = _pid_c(pid_params)
    lib = N.lib()
    dev = plan.device
    max_saves = max_steps // save_every + 1
    ws = workspace(lib.mjx_imex2d_ws_bytes(grid.ny, grid.nx, len(names), plan.code), dev, "imex")
    y_final = torch.empty_like(interior)
    t_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    dt_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    if save_y_history == "host":  # streamed to pinned host memory by the history kernel
        y_hist = torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype,
                             pin_memory=True)
    elif save_y_history:
        y_hist = torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype, device=dev)
    else:
        y_hist = None
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


def _adaptive_imex_general(model, interior, plan, diffusivities, use_strang, t0, t_end, dt0, max_steps,
                           cfl_params, pid_params, save_every, save_y_history, max_attempts):
    """The adaptive IMEX loop on a grid of any size: the same step doubling, error norm, PI
    controller with the IMEX CFL limit and accept/reject rules as the device loop
    (stepping.py:1146-1371), with the native general-size steps; the controller runs on the
    host (one scalar read per attempt)."""
    from moljax_gb300.core.dt_policy import ControllerState, imex_cfl_dt, propose_dt_imex
    from moljax_gb300.core.utils import StatusCode as S
    grid, names = model.grid, model.field_names
    order = 2 if use_strang else 1
    dev = interior.device
    dt = min(float(dt0), imex_cfl_dt(grid, model.params, cfl_params))
    max_saves = max_steps // save_every + 1
    t_hist = torch.zeros(max_saves, dtype=torch.float64, device=dev)
    dt_hist = torch.zeros(max_saves, dtype=torch.float64, device=dev)
    if save_y_history == "host":
        y_hist = torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype, pin_memory=True)
    elif save_y_history:
        y_hist = torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype, device=dev)
    else:
        y_hist = None
    t_hist[0] = t0
    if y_hist is not None:
        y_hist[0].copy_(interior)
    lib = N.lib()
    ews = workspace(lib.mjx_error_norm_ws_bytes(), dev, "errnorm")
    res = (C.c_double * 2)()
    cap = max_attempts if max_attempts and max_attempts > 0 else 20 * max_steps + 1000

    def step(x, h):
        return _imex_interior_general(model, plan, x, h, diffusivities, use_strang)

    t, y, cs = float(t0), interior, ControllerState(1.0, 1.0, 0)
    write_idx, n_acc, n_rej, status, attempts = 1, 0, 0, S.RUNNING, 0
    while status == S.RUNNING and t < t_end and write_idx < max_saves and attempts < cap:
        attempts += 1
        dtc = min(dt, t_end - t)
        y_full = step(y, dtc)
        y_half = step(step(y, 0.5 * dtc), 0.5 * dtc)
        err = y_half - y_full
        N.check("mjx_scaled_error_norm", lib.mjx_scaled_error_norm(
            N.ptr(err), N.ptr(y_half), err.numel(), N.dtype_code(err.dtype), float(pid_params.atol),
            float(pid_params.rtol), res, N.ptr(ews), ews.numel(), N.stream_ptr(dev)))
        e, finite = max(float(res[0]), 1e-10), res[1] != 0.0
        dt_new, cs_new = propose_dt_imex(grid, model.params, None, t, dtc, e, cs, cfl_params, pid_params, order)
        if e <= 1.0 and finite:
            if n_acc % save_every == 0:
                t_hist[write_idx] = t + dtc
                dt_hist[write_idx - 1] = dtc
                if y_hist is not None:
                    y_hist[write_idx].copy_(y_half)
                write_idx += 1
            t, y, dt, cs = t + dtc, y_half, dt_new, cs_new
            n_acc += 1
        else:
            dt = max(dt_new * 0.5, pid_params.dt_min)
            if dt <= pid_params.dt_min * 1.1:
                status = S.DT_TOO_SMALL
            n_rej += 1
        if not finite:
            status = S.NON_FINITE_VALUES
    if t >= t_end:  # as the device controller ends the loop
        status = S.SUCCESS
    elif write_idx >= max_saves or status == S.RUNNING:
        status = S.MAX_STEPS_REACHED
    padded = stencil.pad_interior(y, grid, model.bc_spec, names, t, model.params)
    y_fin = {n: padded[i] for i, n in enumerate(names)}
    y_history = ({n: y_hist[:, i] for i, n in enumerate(names)} if y_hist is not None else None)
    return AdaptiveResult(t, y_fin, t_hist, y_history, dt_hist, write_idx, n_acc, n_rej, status)


class ImexPlan:
    """Persistent native plan of the mixed-precision adaptive IMEX-Strang loop
    (``mjx_imex_plan_*``): the attempt kernels and controller are captured once into a
    CUDA graph with a conditional while node and every ``run`` replays it, with no
    capture, instantiation or allocation per solve.  Fixed at creation: the grid, the
    native problem (reaction, D, F, k, CFL limit), the PID settings, max_steps and
    save_every; ``run`` takes the state and t0, t_end, dt0.  Runs of one plan must not
    overlap (one thread, one stream at a time)."""

    def __init__(self, grid_plan, prob, pid_params, max_steps: int, save_every: int, nfields: int):
        from moljax_gb300.core.fft_solvers import get_plan
        p = grid_plan
        self.p32 = get_plan(p.ny, p.nx, p.dy, p.dx, p.symbol, torch.float32, p.device)
        self.p64 = get_plan(p.ny, p.nx, p.dy, p.dx, p.symbol, torch.float64, p.device)
        self.device = p.device
        self.max_saves = max_steps // save_every + 1
        lib = N.lib()
        nbytes = lib.mjx_imex_plan_ws_bytes(p.ny, p.nx, nfields, self.max_saves)
        self.ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        self._prob, self._pid = prob, _pid_c(pid_params)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check("mjx_imex_plan_create", lib.mjx_imex_plan_create(
                C.byref(h), N.ptr(self.p32.buf), N.ptr(self.p64.buf), C.byref(self.p32.cgrid), C.byref(prob),
                C.byref(self._pid), int(max_steps), int(save_every), N.ptr(self.ws), nbytes))
        self._h = h

    def run(self, interior, t0: float, t_end: float, dt0: float):
        """(y_final interior, t history, dt history, native result) of one solve."""
        y_final = torch.empty_like(interior)
        t_hist = torch.empty(self.max_saves, dtype=torch.float64, device=self.device)
        dt_hist = torch.empty(self.max_saves, dtype=torch.float64, device=self.device)
        res = N.AdaptiveResultC()
        dp = C.POINTER(C.c_double)
        N.check("mjx_imex_plan_run", N.lib().mjx_imex_plan_run(
            self._h, N.dtype_code(interior.dtype), float(t0), float(t_end), float(dt0), N.ptr(interior),
            N.ptr(y_final), C.cast(C.c_void_p(t_hist.data_ptr()), dp), C.cast(C.c_void_p(dt_hist.data_ptr()), dp),
            C.byref(res), N.stream_ptr(self.device)))
        return y_final, t_hist, dt_hist, res

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            N.lib().mjx_imex_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


_imex_plans: "OrderedDict" = None
_IMEX_PLAN_CACHE = 16  # plans kept per process (least recently used dropped first)


def _cached_imex_plan(grid_plan, prob, pid_params, max_steps, save_every, nfields):
    """The persistent plan for this problem (one per host thread: runs must not overlap)."""
    global _imex_plans
    import threading
    from collections import OrderedDict
    if _imex_plans is None:
        _imex_plans = OrderedDict()
    key = (threading.get_ident(), str(grid_plan.device), grid_plan.ny, grid_plan.nx, grid_plan.dy, grid_plan.dx,
           grid_plan.symbol, nfields, bytes(prob), bytes(_pid_c(pid_params)), int(max_steps), int(save_every))
    plan = _imex_plans.get(key)
    if plan is None:
        plan = ImexPlan(grid_plan, prob, pid_params, max_steps, save_every, nfields)
        _imex_plans[key] = plan
        while len(_imex_plans) > _IMEX_PLAN_CACHE:
            _imex_plans.popitem(last=False)[1].close()
    else:
        _imex_plans.move_to_end(key)
    return plan


def _adaptive_mixed(model, interior, plan, prob, pid_params, t0, t_end, dt0, max_steps,
                    save_every) -> AdaptiveResult:
    grid = model.grid
    names = model.field_names
    ip = _cached_imex_plan(plan, prob, pid_params, max_steps, save_every, len(names))
    y_final, t_hist, dt_hist, res = ip.run(interior, t0, t_end, dt0)
    padded = stencil.pad_interior(y_final, grid, model.bc_spec, names, res.t_final, model.params)
    y_fin = {n: padded[i] for i, n in enumerate(names)}
    return AdaptiveResult(res.t_final, y_fin, t_hist, None, dt_hist, res.n_saved, res.n_accepted,
                          res.n_rejected, res.status)


# ------------------------------------------------------------------ explicit steppers
_EXPLICIT = {IntegratorType.EULER: 0, IntegratorType.SSPRK3: 1, IntegratorType.RK4: 2}


def explicit_problem(model, method: int = 2, cfl_params: Optional[CFLParams] = None,
                     t: float = 0.0, max_attempts: int = 0) -> "N.ExplicitProblemC":
    """Native description of a built-in model for the explicit steppers: reaction,
    per-field D, advection (metadata 'advection': 1 upwind, 2 central; params vx, vy),
    per-field BC kinds and side values at time t, heisenberg_cfl_dt."""
    from moljax_gb300.core.bc import side_values
    from moljax_gb300.core.dt_policy import heisenberg_cfl_dt
    names = model.field_names
    if len(names) > 4:
        raise NotImplementedError("at most 4 fields per native explicit call")
    p = N.ExplicitProblemC()
    p.reaction = model.reaction_kind
    p.nfields = len(names)
    D = model.diffusivities()
    for i, n in enumerate(names):
        p.D[i] = float(D.get(n, 0.0))
        spec = model.bc_spec[n]
        p.bc_kind[i] = int(spec.kind)
        for j, v in enumerate(side_values(spec, model.grid, t, model.params)):
            p.bc_values[4 * i + j] = float(v)
    p.F = float(model.params.get("F", 0.0))
    p.k = float(model.params.get("k", 0.0))
    p.r = float(model.params.get("r", 0.0))
    p.advection = int(model.metadata.get("advection", 0))
    p.vx = float(model.params.get("vx", 0.0)) if p.advection else 0.0
    p.vy = float(model.params.get("vy", 0.0)) if p.advection else 0.0
    p.method = int(method)
    if p.reaction == N.REACT_KINETICS:
        p.kin = model.nonlinear_ops[0].native[1]
    p.dt_cfl = heisenberg_cfl_dt(model.grid, model.params, cfl_params or CFLParams())
    p.max_attempts = int(max_attempts)
    return p


def _explicit_steps(model, y, t, dt, method, n_steps=1):
    grid = model.grid
    names = model.field_names
    interior = stencil.unpad(stencil.stack(y, names), grid)
    N.require_cuda(interior)
    prob = explicit_problem(model, method, t=t)
    lib = N.lib()
    code = N.dtype_code(interior.dtype)
    ws = workspace(lib.mjx_explicit_ws_bytes(grid.ny, grid.nx, len(names), code), interior.device,
                   "explicit")
    out = torch.empty_like(interior)
    N.check("mjx_explicit_integrate2d", lib.mjx_explicit_integrate2d(
        C.byref(N.Grid2DC(grid.ny, grid.nx, grid.dy, grid.dx)), code, C.byref(prob), float(dt),
        int(n_steps), N.ptr(interior), N.ptr(out), N.ptr(ws), ws.numel(),
        N.stream_ptr(interior.device)))
    padded = stencil.pad_interior(out, grid, model.bc_spec, names, t + n_steps * dt, model.params)
    return {n: padded[i] for i, n in enumerate(names)}


def euler_step(model, y, t, dt):
    """y + dt F(y) (moljax/core/stepping.py:64-84); ghosts refilled from the BCs."""
    return _explicit_steps(model, y, t, dt, 0)


def ssprk3_step(model, y, t, dt):
    """Shu-Osher SSPRK3 (moljax/core/stepping.py:87-123)."""
    return _explicit_steps(model, y, t, dt, 1)


def rk4_step(model, y, t, dt):
    """Classical RK4 (moljax/core/stepping.py:126-163)."""
    return _explicit_steps(model, y, t, dt, 2)


def _adaptive_explicit(model, y0, t0, t_end, dt0, method, max_steps, cfl_params, pid_params,
                       save_every, save_y_history=True, max_attempts=0):
    grid = model.grid
    names = model.field_names
    pid_params = pid_params or PIDParams()
    interior = stencil.unpad(stencil.stack(y0, names), grid)
    N.require_cuda(interior)
    from moljax_gb300.core import autotune
    autotune.tune_stencil_once(model, interior.dtype)  # tile height of the stage kernel, once per size
    prob = explicit_problem(model, _EXPLICIT[method], cfl_params, t0, max_attempts)
    lib = N.lib()
    dev = interior.device
    code = N.dtype_code(interior.dtype)
    ws = workspace(lib.mjx_explicit_ws_bytes(grid.ny, grid.nx, len(names), code), dev, "explicit")
    max_saves = max_steps // save_every + 1
    y_final = torch.empty_like(interior)
    t_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    dt_hist = torch.empty(max_saves, dtype=torch.float64, device=dev)
    if save_y_history == "host":
        y_hist = torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype,
                             pin_memory=True)
    elif save_y_history:
        y_hist = torch.empty((max_saves,) + tuple(interior.shape), dtype=interior.dtype, device=dev)
    else:
        y_hist = None
    pid = _pid_c(pid_params)
    res = N.AdaptiveResultC()
    N.check("mjx_explicit_adaptive2d", lib.mjx_explicit_adaptive2d(
        C.byref(N.Grid2DC(grid.ny, grid.nx, grid.dy, grid.dx)), code, C.byref(prob), C.byref(pid),
        float(t0), float(t_end), float(dt0), int(max_steps), int(save_every), N.ptr(interior),
        N.ptr(y_final), C.cast(C.c_void_p(t_hist.data_ptr()), C.POINTER(C.c_double)),
        C.cast(C.c_void_p(dt_hist.data_ptr()), C.POINTER(C.c_double)), N.ptr(y_hist),
        N.ptr(ws), ws.numel(), C.byref(res), N.stream_ptr(dev)))
    padded = stencil.pad_interior(y_final, grid, model.bc_spec, names, res.t_final, model.params)
    y_fin = {n: padded[i] for i, n in enumerate(names)}
    y_history = ({n: y_hist[:, i] for i, n in enumerate(names)} if y_hist is not None else None)
    return AdaptiveResult(res.t_final, y_fin, t_hist, y_history, dt_hist, res.n_saved,
                          res.n_accepted, res.n_rejected, res.status)


# ------------------------------------------------------------------ implicit steppers
_IMPLICIT = {IntegratorType.BE: 3, IntegratorType.CN: 4, IntegratorType.BDF2: 5}


def _require_vardiff(model):
    if model.metadata.get("kind") != "vardiff":
        raise NotImplementedError(
            "the native implicit steppers are built for the variable-diffusion model "
            "(create_variable_diffusion_model); for other residuals call newton_krylov_solve")


def _nk_setup(model, nk_params):
    import ctypes as Cc
    from moljax_gb300.core.fft_solvers import get_plan
    from moljax_gb300.core.newton_krylov import NKParams, _cparams
    _require_vardiff(model)
    p = nk_params or NKParams()
    g = model.grid
    a, b, c = model.metadata["abc"]
    return p, _cparams(p), (Cc.c_double * 3)(a, b, c), g


def _interior64(model, y):
    u = y["u"]
    N.require_cuda(u)
    return stencil.unpad(u[None], model.grid)[0].to(torch.float64).contiguous()


def _padded(model, interior, like):
    out = torch.zeros(like.shape, dtype=torch.float64, device=interior.device)
    out[model.grid.interior_slice] = interior
    out = stencil.apply_bc({"u": out}, model.grid, model.bc_spec, 0.0, model.params)["u"]
    return out.to(like.dtype)


def _implicit_step(model, y, y_prev, dt, dt_prev, method, nk_params, be_guess):
    from moljax_gb300.core.fft_solvers import get_plan, workspace
    from moljax_gb300.core.newton_krylov import NKStats
    p, cp, abc, g = _nk_setup(model, nk_params)
    yn = _interior64(model, y)
    yp = _interior64(model, y_prev) if y_prev is not None else yn
    n = g.nx
    plan2 = get_plan(2 * n, 2 * n, g.dy, g.dx, "fd", torch.float32, yn.device)
    lib = N.lib()
    ws = workspace(lib.mjx_nk_vardiff_ws_bytes(n, p.gmres_restart), plan2.device, "nk")
    out = torch.empty_like(yn)
    st = (C.c_int * 3)()
    rn = C.c_double(0.0)
    N.check("mjx_nk_vardiff_step2d", lib.mjx_nk_vardiff_step2d(
        N.ptr(plan2.buf), n, float(g.dy), float(g.dx), abc, int(method), float(dt), float(dt_prev),
        int(be_guess == "previous"), C.byref(cp), N.ptr(yn), N.ptr(yp), N.ptr(out), st,
        C.byref(rn), N.ptr(ws), ws.numel(), N.stream_ptr(plan2.device)))
    return ({"u": _padded(model, out, y["u"])},
            NKStats(bool(st[2]), int(st[0]), int(st[1]), float(rn.value)))


def be_step(model, y, t, dt, preconditioner=None, nk_params=None, *, be_guess: str = "euler"):
    """Backward Euler y_{n+1} = y_n + dt F(y_{n+1}) (moljax/core/stepping.py:170-214).

    Newton-Krylov on the native solver; the explicit-Euler initial guess of the
    reference, or y_n with ``be_guess="previous"``.  The solver always applies its
    own (alpha0 I - beta Dbar Lap_D)^-1 preconditioner (``preconditioner`` is
    accepted for the reference signature; it changes GMRES counts, not the root).
    Returns (y_new, NKStats).
    """
    return _implicit_step(model, y, None, dt, dt, 3, nk_params, be_guess)


def cn_step(model, y, t, dt, preconditioner=None, nk_params=None, *, be_guess: str = "euler"):
    """Crank-Nicolson y_{n+1} = y_n + dt/2 (F(y_n) + F(y_{n+1})) (stepping.py:217-260)."""
    return _implicit_step(model, y, None, dt, dt, 4, nk_params, be_guess)


def bdf2_step(model, y, y_prev, t, dt, dt_prev, preconditioner=None, nk_params=None):
    """Variable-step BDF2 with the reference coefficients (stepping.py:263-310,
    newton_krylov.py:406-448); guess 2 y_n - y_{n-1}."""
    return _implicit_step(model, y, y_prev, dt, dt_prev, 5, nk_params, "euler")


def integrate_fixed_dt(model, y0, t0, t_end, dt, method=IntegratorType.RK4, save_every: int = 1,
                       preconditioner=None, nk_params=None, *, be_guess: str = "euler"):
    """moljax/core/stepping.py:1028-1139 for the implicit methods: int((t_end-t0)/dt)+1
    fixed steps (BDF2 takes a BE first step); returns (t_history, y_history, y_final)
    with every step's padded state, as the reference's scan outputs."""
    method = IntegratorType(int(method))
    n_steps = int((t_end - t0) / dt) + 1
    if method in _EXPLICIT:
        y, t = y0, t0
        ts, ys = [], []
        for _ in range(n_steps):
            y = _explicit_steps(model, y, t, dt, _EXPLICIT[method])
            t = t + dt
            ts.append(t)
            ys.append(y)
        return (torch.tensor(ts, dtype=torch.float64),
                {k: torch.stack([s_[k] for s_ in ys]) for k in y0}, y)
    if method not in _IMPLICIT:
        raise NotImplementedError(f"{method.name}: use integrate_imex_fixed_dt for IMEX methods")
    y, y_prev, t = y0, y0, t0
    ts, ys = [], []
    for step in range(n_steps):
        if method == IntegratorType.BE or (method == IntegratorType.BDF2 and step < 1):
            y_new, _ = be_step(model, y, t, dt, preconditioner, nk_params, be_guess=be_guess)
        elif method == IntegratorType.CN:
            y_new, _ = cn_step(model, y, t, dt, preconditioner, nk_params, be_guess=be_guess)
        else:
            y_new, _ = bdf2_step(model, y, y_prev, t, dt, dt, preconditioner, nk_params)
        y_prev, y, t = y, y_new, t + dt
        ts.append(t)
        ys.append(y)
    return (torch.tensor(ts, dtype=torch.float64),
            {k: torch.stack([s[k] for s in ys]) for k in y0}, y)


def _adaptive_implicit(model, y0, t0, t_end, dt0, method, max_steps, pid_params, nk_params,
                       save_every, be_guess, save_y_history=True, attempt_log=None):
    from moljax_gb300.core.fft_solvers import get_plan, workspace
    pid_params = pid_params or PIDParams()
    p, cp, abc, g = _nk_setup(model, nk_params)
    u0 = _interior64(model, y0)
    n = g.nx
    dev = u0.device
    plan2 = get_plan(2 * n, 2 * n, g.dy, g.dx, "fd", torch.float32, dev)
    lib = N.lib()
    ws = workspace(lib.mjx_nk_vardiff_ws_bytes(n, p.gmres_restart), plan2.device, "nk")
    max_saves = max_steps // save_every + 1
    t_hist = (C.c_double * max_saves)()
    dt_hist = (C.c_double * max_saves)()
    y_hist = (torch.empty((max_saves, n, n), dtype=torch.float64, device=dev)
              if save_y_history else None)
    y_final = torch.empty_like(u0)
    tot = (C.c_int * 3)()
    log_cap = 20 * max_steps + 1000 if attempt_log is not None else 0
    log = (C.c_double * (6 * max(log_cap, 1)))() if attempt_log is not None else None
    res = N.AdaptiveResultC()
    pid = _pid_c(pid_params)
    N.check("mjx_nk_vardiff_adaptive2d", lib.mjx_nk_vardiff_adaptive2d(
        N.ptr(plan2.buf), n, float(g.dy), float(g.dx), abc, _IMPLICIT[method], C.byref(pid),
        float(t0), float(t_end), float(dt0), int(max_steps), int(save_every),
        int(be_guess == "previous"), C.byref(cp), N.ptr(u0), N.ptr(y_final), t_hist, dt_hist,
        N.ptr(y_hist), tot, log, int(log_cap), C.byref(res), N.ptr(ws), ws.numel(),
        N.stream_ptr(dev)))
    if attempt_log is not None:  # (t, dt, err, converged, newton_iters, accepted) per attempt
        attempt_log.extend(tuple(log[6 * i:6 * i + 6]) for i in range(res.n_attempts))
    y_fin = {"u": _padded(model, y_final, y0["u"])}
    th = torch.tensor(list(t_hist), dtype=torch.float64)
    dth = torch.tensor(list(dt_hist), dtype=torch.float64)
    return AdaptiveResult(res.t_final, y_fin, th, {"u": y_hist} if y_hist is not None else None,
                          dth, res.n_saved, res.n_accepted, res.n_rejected, res.status)


def adaptive_integrate(model, y0=None, t0: float = 0.0, t_end: Optional[float] = None,
                       dt0: float = 1.0, method: int = IntegratorType.RK4, max_steps: int = 10000,
                       cfl_params: Optional[CFLParams] = None,
                       pid_params: Optional[PIDParams] = None, preconditioner=None,
                       nk_params=None, save_every: int = 1, *, t_span=None, integrator=None,
                       rtol: Optional[float] = None, atol: Optional[float] = None, **kw):
    """Reference form (stepping.py:723-1021) or README form (README.md:75-80).

    IMEX_STRANG and IMEX_EULER route to ``adaptive_integrate_imex`` (the
    reference's real IMEX driver; the reference's own adaptive_integrate lets
    both fall through to its BDF2 branch, stepping.py:864-877).  Other methods
    are dispatched to their native drivers as they are built; unbuilt ones
    raise NotImplementedError.
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
        from moljax_gb300.core.fft_integrators import etd_integrate_model
        y, tf = etd_integrate_model(model, y0, t0, t_end, dt0, kw.pop("symbol", "fd"))
        n = int(round((tf - t0) / dt0))
        return AdaptiveResult(tf, y, torch.tensor([t0, tf], dtype=torch.float64), None,
                              torch.tensor([dt0], dtype=torch.float64), 2, n, 0, 0)
    if method in _EXPLICIT:
        return _adaptive_explicit(model, y0, t0, t_end, dt0, method, max_steps, cfl_params,
                                  pid_params, save_every, kw.pop("save_y_history", True),
                                  kw.pop("max_attempts", 0))
    if method in _IMPLICIT:
        return _adaptive_implicit(model, y0, t0, t_end, dt0, method, max_steps, pid_params,
                                  nk_params, save_every, kw.pop("be_guess", "euler"),
                                  kw.pop("save_y_history", True), kw.pop("attempt_log", None))
    if method in (IntegratorType.IMEX_STRANG, IntegratorType.IMEX_EULER):
        return adaptive_integrate_imex(model, y0, t0, t_end, dt0, None, None,
                                       method == IntegratorType.IMEX_STRANG, max_steps,
                                       cfl_params, pid_params, save_every, **kw)
    raise NotImplementedError(f"{method.name} adaptive driver is not built on the GPU path")


# ------------------------------------------------------------------ step-doubling helpers
class AdaptiveState(NamedTuple):
    """moljax/core/stepping.py:683-707: the loop state of the reference's adaptive
    while_loop.  The native drivers keep it on the device (DevState); this record is the
    host-side mirror for callers that build their own loops."""
    t: float
    y: Dict[str, torch.Tensor]
    dt: float
    y_prev: Optional[Dict[str, torch.Tensor]]
    dt_prev: float
    step_count: int
    controller: object
    t_history: torch.Tensor
    y_history: Optional[Dict[str, torch.Tensor]]
    dt_history: torch.Tensor
    write_idx: int
    n_accepted: int
    n_rejected: int
    status: int


def _sub(a, b):
    return {k: a[k] - b[k] for k in a}


def estimate_error_doubling(model, y, t, dt, step_fn):
    """(y_half2, y_half2 - y_full) from one step of dt and two of dt/2 (stepping.py:502-536)."""
    y_full = step_fn(model, y, t, dt)
    y_half2 = step_fn(model, step_fn(model, y, t, dt / 2.0), t + dt / 2.0, dt / 2.0)
    return y_half2, _sub(y_half2, y_full)


def estimate_error_implicit(model, y, t, dt, y_be, y_cn):
    """y_cn - y_be (stepping.py:539-563)."""
    return _sub(y_cn, y_be)


def estimate_error_imex_doubling(model, y, t, dt, fft_cache, diffusivities, use_strang: bool = True):
    """Step doubling with IMEX-Strang (or IMEX-Euler) steps (stepping.py:566-608); each step
    is one native fused call.  The adaptive drivers fuse the three steps of an attempt and
    the error norm into one pass sequence instead."""
    fn = imex_strang_step if use_strang else imex_euler_step
    return estimate_error_doubling(model, y, t, dt,
                                   lambda m, yy, tt, h: fn(m, yy, tt, h, fft_cache, diffusivities))


_EXPLICIT_STEPS = {0: "euler_step", 1: "ssprk3_step", 2: "rk4_step"}


def step_explicit(model, y, t, dt, method: int):
    """Euler / SSPRK3 / RK4 by index 0 / 1 / 2 (stepping.py:615-643)."""
    return globals()[_EXPLICIT_STEPS[int(method)]](model, y, t, dt)


def step_explicit_with_error(model, y, t, dt, method: int):
    """Step doubling with the explicit method of index 0 / 1 / 2 (stepping.py:646-676)."""
    fn = globals()[_EXPLICIT_STEPS[int(method)]]
    return estimate_error_doubling(model, y, t, dt, fn)


def imex_ssprk2_step(model, y, t, dt, fft_cache, diffusivities):
    """IMEX-SSPRK2 (stepping.py:438-495): y1 = H(dt)(y + dt N(y)), y2 = H(dt)(y1 + dt N(y1)),
    y_new = (y + y2)/2, the BCs applied after each stage.  y + dt N(y) is the native
    Euler reaction kernel (on the interiors; every ghost is refilled by the BCs), H the
    Helmholtz pass of the grid's spectral plan (any size)."""
    from moljax_gb300.core.fft_solvers import apply_diffusion_inverse_fft
    grid = model.grid
    names = model.field_names
    rx, F, k, r = _reaction_args(model)

    def stage(z, tt):
        inter = stencil.unpad(stencil.stack(z, names), grid)
        out = torch.empty_like(inter)
        N.check("mjx_reaction_step2d", N.lib().mjx_reaction_step2d(
            N.ptr(inter), N.ptr(out), len(names), inter[0].numel(), rx, F, k, r, float(dt), 1,
            N.dtype_code(out.dtype), N.stream_ptr(out.device)))
        rhs = dict(z)
        for i, n in enumerate(names):
            rr = z[n].clone()
            rr[grid.interior_slice] = out[i]
            rhs[n] = rr
        return model.apply_bcs(apply_diffusion_inverse_fft(rhs, grid, dt, diffusivities, fft_cache), tt)

    y = model.apply_bcs(y, t)
    y1 = stage(y, t + dt)
    y2 = stage(y1, t + dt)
    return model.apply_bcs({k_: 0.5 * y[k_] + 0.5 * y2[k_] for k_ in y}, t + dt)
