"""Exponential time differencing on periodic grids (moljax/core/fft_integrators.py).

Every integrator here runs natively (``mjx_etd_integrate2d``): one column pass
per stage fuses the forward FFT along y, the stage combination with FP64-built
coefficient tables and the inverse FFT; one row pass per stage fuses c2r, the
nonlinear term and r2c.  Steps of one kind are captured once in a CUDA graph
and replayed.

* ``etd1_step`` / ``etd2_step`` / ``etdrk4_step`` / ``etd_integrate`` keep the
  library signatures (fft_integrators.py:119-393) on interior fields, 1D
  ``(n,)`` or 2D ``(ny, nx)``.  ``nonlinear_rhs`` must be a native term: a
  ``NativeNonlinear`` (Gray-Scott, logistic, zero) or a MOLModel with a
  Gray-Scott or Fisher-KPP reaction.  The library ETDRK4 evaluates the later
  stages one field at a time (311-327) and so cannot couple u and v; here the
  stages are evaluated on all fields together, which is the same for the
  uncoupled logistic term.  Fields without a linear operator get L = 0, for
  which the ETD1, ETD2 and ETDRK4 updates reduce to the library's Euler, AB2 and
  RK4 fallbacks.
* ``etdrk4_gray_scott`` runs the coupled Gray-Scott ETDRK4 of the benchmark
  (benchmarks/benchmark_gray_scott.py:336-417) on a padded MOLModel state, with
  the 32-point contour coefficients.

1D fields are carried as two identical rows of a (2, n) grid whose symbol has
no y part, so each row is exactly the 1D problem.
"""

from __future__ import annotations

import ctypes as C
import math
from typing import Dict, NamedTuple, Optional

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core import stencil
from moljax_gb300.core.fft_solvers import get_plan, workspace

_coeff_key = {}

METHODS = {"etd1": N.ETD_1, "etd2": N.ETD_2, "etdrk4": N.ETD_RK4}


class ETDStepResult(NamedTuple):
    """fft_integrators.py:31-35."""
    state: Dict[str, torch.Tensor]
    t: float
    diagnostics: dict


def _symbol_code(symbol):
    return {"fd": N.SYMBOL_FD, "spectral": N.SYMBOL_SPECTRAL}[symbol]


class NativeNonlinear:
    """A nonlinear term N(u) that the native row pass evaluates.

    ``NativeNonlinear.gray_scott(F, k)``: (-u v^2 + F (1 - u), u v^2 - (F + k) v)
    on fields u, v (operators.py:655-667); ``NativeNonlinear.logistic(r)``:
    r u (1 - u) on each field (operators.py:680-705); ``NativeNonlinear.zero()``.
    Calling it as ``nonlinear_rhs(state, t)`` evaluates N on the GPU.
    """

    def __init__(self, kind: int, F: float = 0.0, k: float = 0.0, r: float = 0.0):
        self.kind, self.F, self.k, self.r = int(kind), float(F), float(k), float(r)

    @classmethod
    def gray_scott(cls, F: float, k: float) -> "NativeNonlinear":
        return cls(N.REACT_GRAY_SCOTT, F=F, k=k)

    @classmethod
    def logistic(cls, r: float) -> "NativeNonlinear":
        return cls(N.REACT_FISHER, r=r)

    @classmethod
    def zero(cls) -> "NativeNonlinear":
        return cls(N.REACT_NONE)

    @classmethod
    def of(cls, obj) -> "NativeNonlinear":
        if isinstance(obj, NativeNonlinear):
            return obj
        if hasattr(obj, "reaction_kind"):  # a MOLModel
            kind = obj.reaction_kind
            p = obj.params
            return cls(kind, F=p.get("F", 0.0), k=p.get("k", 0.0), r=p.get("r", 1.0))
        raise NotImplementedError(
            "the native ETD path needs a native nonlinear term (NativeNonlinear or a MOLModel with "
            "a Gray-Scott or Fisher-KPP reaction); arbitrary Python callables are not run")

    def __call__(self, state: Dict[str, torch.Tensor], t: float = 0.0) -> Dict[str, torch.Tensor]:
        """N on the fields (any shape), one pointwise native kernel."""
        names = _field_order(state, self)
        y = torch.stack([state[n] for n in names]).contiguous()
        N.require_cuda(y)
        out = torch.empty_like(y)
        N.check("mjx_reaction_step2d", N.lib().mjx_reaction_step2d(
            N.ptr(y), N.ptr(out), len(names), y[0].numel(), self.kind, self.F, self.k, self.r, 0.0, 2,
            N.dtype_code(y.dtype), N.stream_ptr(y.device)))
        return {n: out[i] for i, n in enumerate(names)}


def _field_order(state, nl: NativeNonlinear):
    names = list(state.keys())
    if nl.kind == N.REACT_GRAY_SCOTT:
        if set(names) != {"u", "v"}:
            raise ValueError("the Gray-Scott term acts on fields 'u' and 'v'")
        return ["u", "v"]
    return names


def _pack(state, names):
    """Stack interior fields to (nf, ny, nx); 1D fields become two identical rows."""
    f0 = state[names[0]]
    if f0.ndim == 1:
        return torch.stack([torch.stack([state[n], state[n]]) for n in names]).contiguous(), False
    if f0.ndim != 2:
        raise ValueError("fields must be 1D (n,) or 2D (ny, nx) interior arrays")
    return torch.stack([state[n] for n in names]).contiguous(), True


def _unpack(y, names, is2d):
    if is2d:
        return {n: y[i] for i, n in enumerate(names)}
    return {n: y[i, 0].clone() for i, n in enumerate(names)}


def _grid_of(state, names, linear_ops):
    """(ny, nx, dy, dx, symbol flags) of the packed fields."""
    f0 = state[names[0]]
    op = next((linear_ops[n] for n in names if linear_ops and n in linear_ops), None)
    if f0.ndim == 1:
        n = f0.shape[0]
        dx = op.grid.dx if op is not None else 1.0 / n
        return (2, n, dx, dx), N.SYMBOL_FD | N.SYMBOL_X_ONLY
    ny, nx = f0.shape
    if op is not None:
        return (ny, nx, op.grid.dy, op.grid.dx), N.SYMBOL_FD
    return (ny, nx, 1.0 / ny, 1.0 / nx), N.SYMBOL_FD


def _run(y: torch.Tensor, grid, symbol: int, D, nl: NativeNonlinear, method: int, coeffs: int,
         dt: float, n_steps: int, nprev: Optional[torch.Tensor] = None, want_n: bool = False,
         f2_factor: float = 2.0, tag: str = "etd"):
    """n_steps native ETD steps of packed fields y (nf, ny, nx); returns (y_out, n_out).
    Each workspace tag keeps its own coefficient tables (one per step size in use)."""
    nf = y.shape[0]
    if nf > 2:
        raise NotImplementedError("the native ETD path takes one or two fields per call")
    ny, nx, dy, dx = grid
    plan = get_plan(ny, nx, dy, dx, "fd", y.dtype, y.device)
    if getattr(plan, "general", False):
        return _run_general(plan, y, grid, symbol, D, nl, method, coeffs, dt, n_steps, nprev, want_n, f2_factor)
    lib = N.lib()
    ws = workspace(lib.mjx_etdrk4_ws_bytes(ny, nx, plan.code), plan.device, tag)
    pb = N.ETDProblemC()
    pb.method, pb.coeffs, pb.symbol, pb.reaction, pb.nfields = method, coeffs, symbol, nl.kind, nf
    pb.D[0] = float(D[0])
    pb.D[1] = float(D[1] if nf > 1 else 0.0)
    pb.F, pb.k, pb.r, pb.dt, pb.f2_factor = nl.F, nl.k, nl.r, float(dt), float(f2_factor)
    key = (ny, nx, dy, dx, symbol, y.dtype, tuple(pb.D), float(dt), method, coeffs, float(f2_factor), nf,
           ws.data_ptr())
    recompute = int(_coeff_key.get((str(plan.device), tag)) != key)
    _coeff_key[(str(plan.device), tag)] = key
    out = torch.empty_like(y)
    n_out = torch.empty_like(y) if want_n else None
    cg = N.Grid2DC(ny, nx, dy, dx)
    if nprev is not None:
        nprev = nprev.to(y.dtype).contiguous()
    N.check("mjx_etd_integrate2d", lib.mjx_etd_integrate2d(
        N.ptr(plan.buf), C.byref(cg), plan.code, C.byref(pb), int(n_steps), N.ptr(y),
        N.ptr(nprev) if nprev is not None else None, N.ptr(out), N.ptr(n_out) if want_n else None,
        N.ptr(ws), ws.numel(), recompute, N.stream_ptr(plan.device)))
    return out, n_out


# ------------------------------------------------------------------ grids of any size
def _phi_ref(z: torch.Tensor):
    """phi1, phi2, phi3 as fft_integrators.py:39-78 evaluates them (Taylor below |z| = 1e-4)."""
    small = z.abs() < 1e-4
    zs = torch.where(small, torch.ones_like(z), z)  # keeps the unused branch finite
    ez = torch.exp(z)
    p1 = torch.where(small, 1.0 + z / 2.0 + z ** 2 / 6.0 + z ** 3 / 24.0, (ez - 1.0) / zs)
    p2 = torch.where(small, 0.5 + z / 6.0 + z ** 2 / 24.0 + z ** 3 / 120.0, (ez - 1.0 - z) / (zs * zs))
    p3 = torch.where(small, 1.0 / 6.0 + z / 24.0 + z ** 2 / 120.0 + z ** 3 / 720.0,
                     (ez - 1.0 - z - z ** 2 / 2.0) / (zs * zs * zs))
    return p1, p2, p3


def _symbol_full(ny, nx, dy, dx, symbol, device):
    """The Laplacian symbol on the full (ny, nx) spectrum in FFT order (FD or spectral;
    with MJX_SYMBOL_X_ONLY no y part)."""
    kind = symbol & 1
    kx = 2 * math.pi * torch.fft.fftfreq(nx, d=dx, dtype=torch.float64, device=device)
    ky = 2 * math.pi * torch.fft.fftfreq(ny, d=dy, dtype=torch.float64, device=device)
    if kind == N.SYMBOL_FD:
        lx, ly = (2.0 * torch.cos(kx * dx) - 2.0) / dx ** 2, (2.0 * torch.cos(ky * dy) - 2.0) / dy ** 2
    else:
        lx, ly = -kx ** 2, -ky ** 2
    if symbol & N.SYMBOL_X_ONLY:
        ly = torch.zeros_like(ly)
    return ly[:, None] + lx[None, :]


def _etd_tables(lam, Df, dt, method, coeffs, f2_factor):
    """Per-field coefficient tables on the full spectrum: ETD1/ETD2 (E, dt phi1, dt phi2);
    ETDRK4 (E, E2, Q, f1, f2, f3) from the phi functions or the 32-point contour mean."""
    z = dt * Df * lam
    if method != N.ETD_RK4:
        p1, p2, _ = _phi_ref(z)
        return torch.exp(z), dt * p1, dt * p2
    if coeffs == N.ETD_COEFF_PHI:
        p1, p2, p3 = _phi_ref(z)
        h1, _, _ = _phi_ref(z / 2.0)
        return (torch.exp(z), torch.exp(z / 2.0), dt / 2.0 * h1, dt * (p1 - 3.0 * p2 + 4.0 * p3),
                dt * (2.0 * p2 - 4.0 * p3), dt * (-p2 + 4.0 * p3))
    M = 32
    r = torch.exp(1j * math.pi * (torch.arange(1, M + 1, dtype=torch.float64, device=lam.device) - 0.5) / M)
    LR = z.to(torch.complex128)[..., None] + r
    mean = lambda x: torch.real(x.mean(dim=-1))  # noqa: E731
    Q = dt * mean((torch.exp(LR / 2) - 1) / LR)
    f1 = dt * mean((-4 - LR + torch.exp(LR) * (4 - 3 * LR + LR ** 2)) / LR ** 3)
    f2 = dt * mean((2 + LR + torch.exp(LR) * (-2 + LR)) / LR ** 3)
    f3 = dt * mean((-4 - 3 * LR - LR ** 2 + torch.exp(LR) * (4 - LR)) / LR ** 3)
    return torch.exp(z), torch.exp(z / 2.0), Q, f1, f2_factor * f2, f3


def _run_general(plan, y, grid, symbol, D, nl, method, coeffs, dt, n_steps, nprev, want_n, f2_factor):
    """ETD steps on a grid of any size: each spectral product real(ifft2(T fft2(x))) is one
    native table-multiplier pass of the general plan, the nonlinear term the pointwise
    reaction kernel; the updates combine the passes as fft_integrators.py:119-341 combine
    the spectra."""
    ny, nx, dy, dx = grid
    nf = y.shape[0]
    lam = _symbol_full(ny, nx, dy, dx, symbol, y.device)
    tabs = [tuple(t.to(y.dtype).contiguous() for t in _etd_tables(lam, float(D[f]), dt, method, coeffs, f2_factor))
            for f in range(nf)]

    def mul(x, idx):  # x (nf, ny, nx): field f times table idx of field f
        return torch.stack([plan.apply(x[f].contiguous(), 1.0, 1.0, N.MULT_TABLE, table=tabs[f][idx])
                            for f in range(nf)])

    def Nf(x):
        out = torch.empty_like(x)
        N.check("mjx_reaction_step2d", N.lib().mjx_reaction_step2d(
            N.ptr(x), N.ptr(out), nf, x[0].numel(), nl.kind, nl.F, nl.k, nl.r, 0.0, 2, N.dtype_code(x.dtype),
            N.stream_ptr(x.device)))
        return out

    u = y.contiguous()
    Np = nprev.contiguous() if nprev is not None else None
    n_out = None
    for i in range(int(n_steps)):
        Nu = Nf(u)
        if want_n and i == n_steps - 1:
            n_out = Nu.clone()
        if method == N.ETD_1 or (method == N.ETD_2 and Np is None):
            u_new = mul(u, 0) + mul(Nu, 1)
        elif method == N.ETD_2:
            u_new = mul(u, 0) + mul(Nu, 1) + mul(Nu - Np, 2)
        else:
            a = mul(u, 1) + mul(Nu, 2)
            Na = Nf(a)
            b = mul(u, 1) + mul(Na, 2)
            Nb = Nf(b)
            c = mul(a, 1) + mul(2.0 * Nb - Nu, 2)
            Nc = Nf(c)
            u_new = mul(u, 0) + mul(Nu, 3) + mul(Na + Nb, 4) + mul(Nc, 5)
        if method == N.ETD_2:
            Np = Nu
        u = u_new
    return u, n_out


def _setup(state, linear_ops, nonlinear_rhs, model=None):
    nl = NativeNonlinear.of(model if model is not None else nonlinear_rhs)
    names = _field_order(state, nl)
    y, is2d = _pack(state, names)
    N.require_cuda(y)
    grid, symbol = _grid_of(state, names, linear_ops or {})
    D = [float(linear_ops[n].D) if linear_ops and n in linear_ops else 0.0 for n in names]
    return nl, names, y, is2d, grid, symbol, D


def _groups(names):
    """Fields go through the native call two at a time: the Gray-Scott pair
    together; the other terms act on each field alone."""
    return [list(range(i, min(len(names), i + 2))) for i in range(0, len(names), 2)]


def _advance(state, dt, linear_ops, nonlinear_rhs, method, n_steps, coeffs=N.ETD_COEFF_PHI,
             N_prev=None, want_n=False, model=None):
    nl, names, y, is2d, grid, symbol, D = _setup(state, linear_ops, nonlinear_rhs, model)
    out = torch.empty_like(y)
    nout = torch.empty_like(y) if want_n else None
    nprev = None
    if N_prev is not None:
        nprev, _ = _pack(N_prev, names)
    for g in _groups(names):
        sl = slice(g[0], g[-1] + 1)
        o, no = _run(y[sl].contiguous(), grid, symbol, [D[i] for i in g], nl, method, coeffs, dt, n_steps,
                     nprev[sl] if nprev is not None else None, want_n)
        out[sl] = o
        if want_n:
            nout[sl] = no
    return _unpack(out, names, is2d), (_unpack(nout, names, is2d) if want_n else None)


def etd1_step(state, t: float, dt: float, linear_ops, nonlinear_rhs, model=None):
    """u_{n+1} = exp(dt L) u_n + dt phi1(dt L) N(u_n) (fft_integrators.py:119-175)."""
    return _advance(state, dt, linear_ops, nonlinear_rhs, N.ETD_1, 1, model=model)[0]


def etd2_step(state, t: float, dt: float, linear_ops, nonlinear_rhs, N_prev=None, model=None):
    """ETD2 (fft_integrators.py:178-249): returns (new_state, N(state)); ETD1 without N_prev."""
    return _advance(state, dt, linear_ops, nonlinear_rhs, N.ETD_2, 1, N_prev=N_prev, want_n=True,
                    model=model)


def etdrk4_step(state, t: float, dt: float, linear_ops, nonlinear_rhs, model=None):
    """Cox-Matthews ETDRK4 with the phi-function coefficients (fft_integrators.py:252-341)."""
    return _advance(state, dt, linear_ops, nonlinear_rhs, N.ETD_RK4, 1, model=model)[0]


def etd_integrate(u0, t_span, dt: float, linear_ops, nonlinear_rhs, method: str = "etd1",
                  save_every: int = 1, model=None):
    """fft_integrators.py:344-393: int((t_end - t_start) / dt) steps, the state saved
    every save_every steps; returns (t_history, state_history).  Steps after the last
    save change nothing that is returned and are not run."""
    if method not in METHODS:
        raise ValueError(f"Unknown method: {method}. Use 'etd1', 'etd2', or 'etdrk4'")
    t0, t1 = t_span
    n_steps = int((t1 - t0) / dt)
    nsave = n_steps // save_every
    t_hist = [t0]
    hist = [u0]
    state, N_prev, t = u0, None, t0
    m = METHODS[method]
    for s in range(nsave):
        more = s + 1 < nsave
        state, n_last = _advance(state, dt, linear_ops, nonlinear_rhs, m, save_every,
                                 N_prev=N_prev if m == N.ETD_2 else None,
                                 want_n=(m == N.ETD_2 and more), model=model)
        N_prev = n_last
        for _ in range(save_every):
            t += dt
        t_hist.append(t)
        hist.append(state)
    return torch.tensor(t_hist, dtype=torch.float64), hist


def batched_fft_matvec(state, linear_ops):
    """L u per field; zeros without an operator (fft_integrators.py:400-420)."""
    return {n: (linear_ops[n].matvec(u) if n in linear_ops else torch.zeros_like(u)) for n, u in state.items()}


def batched_fft_solve(rhs, linear_ops, dt: float):
    """(I - dt L)^-1 per field; unchanged without an operator (fft_integrators.py:423-445)."""
    return {n: (linear_ops[n].solve(u, dt) if n in linear_ops else u) for n, u in rhs.items()}


def batched_fft_exp_matvec(state, linear_ops, dt: float):
    """exp(dt L) u per field; unchanged without an operator (fft_integrators.py:448-470)."""
    return {n: (linear_ops[n].exp_matvec(u, dt) if n in linear_ops else u) for n, u in state.items()}


def stacked_fft_solve_shared_op(rhs, op, dt: float):
    """(I - dt L)^-1 for every field with one shared operator (fft_integrators.py:473-510);
    a shared DiffusionOperator runs all fields through one native pass (four per launch)."""
    from moljax_gb300.core.fft_operators import DiffusionOperator
    names = list(rhs.keys())
    if not names:
        return {}
    if not isinstance(op, DiffusionOperator):
        return {n: op.solve(rhs[n], dt) for n in names}
    x = torch.stack([rhs[n] for n in names]).contiguous()
    plan = op._plan(x.dtype)
    if op.is_1d:
        from moljax_gb300.core.fft_solvers import _apply_1d
        y = _apply_1d(plan, x, op.D, dt, N.MULT_HELMHOLTZ)
    else:
        y = plan.apply(x, op.D, dt, N.MULT_HELMHOLTZ)
    return {n: y[i] for i, n in enumerate(names)}


def imex_euler_step(state, t: float, dt: float, linear_ops, nonlinear_rhs, model=None):
    """(I - dt L) u_{n+1} = u_n + dt N(u_n) (fft_integrators.py:545-585): N by the native
    row pass, the solve by the operator's spectral pass; without an operator, explicit
    Euler."""
    nl = NativeNonlinear.of(model if model is not None else nonlinear_rhs)
    Nn = nl(state, t)
    out = {}
    for n, u in state.items():
        r = u + dt * Nn[n]
        out[n] = linear_ops[n].solve(r, dt) if n in linear_ops else r
    return out


def diffusion_only_etd1(u0: torch.Tensor, t_end: float, dt: float, op) -> torch.Tensor:
    """fft_integrators.py:513-542: max(1, int(t_end/dt)) steps of exp(h L), h = t_end/n."""
    n = max(1, int(t_end / dt))
    h = t_end / n
    u = u0
    for _ in range(n):
        u = op.exp_matvec(u, h)
    return u


def etdrk4_gray_scott(model, y0, dt: float, n_steps: int, symbol: str = "fd",
                      variant: str = "cox-matthews"):
    """Fixed-step coupled ETDRK4 on a Gray-Scott MOLModel (padded state in and out).

    ``variant="cox-matthews"`` is the fourth-order method (the library's
    coefficients, fft_integrators.py:106-113); ``variant="benchmark"``
    reproduces benchmarks/benchmark_gray_scott.py:415, whose final update uses
    f2 (N^a + N^b) without the factor 2 of the Kassam-Trefethen form.
    """
    f2_factor = {"cox-matthews": 2.0, "benchmark": 1.0}[variant]
    if model.reaction_kind != N.REACT_GRAY_SCOTT:
        raise NotImplementedError("etdrk4_gray_scott is the coupled Gray-Scott integrator")
    grid = model.grid
    names = model.field_names
    interior = stencil.unpad(stencil.stack(y0, names), grid)
    D = model.diffusivities()
    nl = NativeNonlinear.of(model)
    out, _ = _run(interior, (grid.ny, grid.nx, grid.dy, grid.dx), _symbol_code(symbol), [D["u"], D["v"]], nl,
                  N.ETD_RK4, N.ETD_COEFF_CONTOUR, dt, n_steps, f2_factor=f2_factor)
    padded = stencil.pad_interior(out, grid, model.bc_spec, names)
    return {n: padded[i] for i, n in enumerate(names)}


def etd_integrate_model(model, y0, t0: float, t_end: float, dt: float, symbol: str = "fd",
                        variant: str = "cox-matthews"):
    """Fixed-step coupled ETDRK4 of a Gray-Scott MOLModel from t0 to t_end:
    n = ceil((t_end - t0)/dt) steps (the benchmark's step count); returns (state, t)."""
    n = int(math.ceil((t_end - t0) / dt - 1e-12))
    return etdrk4_gray_scott(model, y0, dt, n, symbol, variant), t0 + n * dt


def etd_adaptive_integrate(u0, t0: float, t_end: float, dt0: float, linear_ops, nonlinear_rhs,
                           method: str = "etdrk4", pid_params=None, max_steps: int = 10000,
                           save_every: int = 1, model=None, max_attempts: Optional[int] = None):
    """Adaptive ETD1 / ETDRK4 by step doubling (the reference has fixed-step ETD only).

    Each attempt runs one native step of dt and two of dt/2 from the same state (two
    workspaces, so each step size keeps its coefficient tables), takes the scaled
    RMS of their difference with the native error norm, and applies the explicit
    branch of adaptive_integrate (moljax/core/stepping.py:723-1021): PI controller of
    order compute_error_order (1 for ETD1, 4 for ETDRK4, dt_policy.py:178-268),
    halving after a reject, DT_TOO_SMALL / NON_FINITE_VALUES / MAX_STEPS_REACHED.
    No CFL limit applies: the linear part is integrated exactly.  The accepted state
    is the two-half-step result.  Returns an AdaptiveResult (interior fields; no y
    history)."""
    from moljax_gb300.core.dt_policy import (PIDParams, ControllerState, pid_controller_dt,
                                             handle_rejected_step)
    from moljax_gb300.core.fft_solvers import workspace as _ws
    from moljax_gb300.core.stepping import AdaptiveResult
    from moljax_gb300.core.utils import StatusCode as S
    if method not in ("etd1", "etdrk4"):
        raise ValueError("adaptive ETD: method 'etd1' or 'etdrk4' (ETD2 is a multistep method)")
    pid = pid_params or PIDParams()
    order = 1 if method == "etd1" else 4
    m = METHODS[method]
    nl, names, y, is2d, grid, symbol, D = _setup(u0, linear_ops, nonlinear_rhs, model)
    if len(names) > 2:
        raise NotImplementedError("adaptive ETD takes one or two fields")
    lib = N.lib()
    ews = _ws(lib.mjx_error_norm_ws_bytes(), y.device, "errnorm")
    res = (C.c_double * 2)()
    max_saves = max_steps // save_every + 1
    t_hist = torch.zeros(max_saves, dtype=torch.float64)
    dt_hist = torch.zeros(max_saves, dtype=torch.float64)
    t_hist[0] = t0
    t, dt, cs = float(t0), float(dt0), ControllerState(1.0, 1.0, 0)
    write_idx, n_acc, n_rej, status, attempts = 1, 0, 0, S.RUNNING, 0
    while status == S.RUNNING and t < t_end and write_idx < max_saves:
        if max_attempts is not None and attempts >= max_attempts:
            break
        attempts += 1
        dtc = min(dt, t_end - t)
        y_full, _ = _run(y, grid, symbol, D, nl, m, N.ETD_COEFF_PHI, dtc, 1, tag="etd")
        y_half, _ = _run(y, grid, symbol, D, nl, m, N.ETD_COEFF_PHI, 0.5 * dtc, 2, tag="etd_half")
        err = y_half - y_full
        N.check("mjx_scaled_error_norm", lib.mjx_scaled_error_norm(
            N.ptr(err), N.ptr(y_half), err.numel(), N.dtype_code(err.dtype), float(pid.atol),
            float(pid.rtol), res, N.ptr(ews), ews.numel(), N.stream_ptr(y.device)))
        e, finite = max(float(res[0]), 1e-10), res[1] != 0.0
        if e <= 1.0:
            dt_a, cs_new = pid_controller_dt(dtc, e, cs, pid, order)
        else:
            dt_a, cs_new = handle_rejected_step(dtc, e, cs, pid, order)[0], cs
        dt_new = min(max(dt_a, pid.dt_min), pid.dt_max)
        if e <= 1.0 and finite:
            if n_acc % save_every == 0:
                t_hist[write_idx] = t + dtc
                dt_hist[write_idx - 1] = dtc
                write_idx += 1
            t, y, dt, cs = t + dtc, y_half, dt_new, cs_new
            n_acc += 1
        else:
            dt = max(dt_new * 0.5, pid.dt_min)
            if dt <= pid.dt_min * 1.1:
                status = S.DT_TOO_SMALL
            n_rej += 1
        if not finite:
            status = S.NON_FINITE_VALUES
    if t >= t_end:
        status = S.SUCCESS
    elif write_idx >= max_saves:
        status = S.MAX_STEPS_REACHED
    return AdaptiveResult(t, _unpack(y, names, is2d), t_hist, None, dt_hist, write_idx, n_acc, n_rej,
                          status)
