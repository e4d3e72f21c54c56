"""Newton-Krylov (moljax/core/newton_krylov.py drop-in).

Two levels:

* ``integrate_implicit_vardiff`` -- the fused native path (hot path of the
  NK benchmark configuration): fixed-dt BE/CN/BDF2 steps of
  u_t = div((a + b u^2) grad u) - c u^3 with homogeneous Dirichlet ghosts,
  each step solved by ``mjx_nk_vardiff_integrate2d``: FP64 residual, FP32
  hand-written JVP and Krylov vectors, left-preconditioned restarted GMRES with
  the Hessenberg/Givens least squares in FP64 on the GPU, DST preconditioner;
* ``newton_krylov_solve(residual_fn, x0, ...)`` -- the reference signature
  for arbitrary Python residuals (newton_krylov.py:171-359): same Newton /
  backtracking semantics, exact JVP by torch forward-mode AD (the counterpart
  of jax.jvp) and a restarted GMRES on torch tensors.  This generic form runs
  user callables and is not the fused path.
"""

from __future__ import annotations

import ctypes as C
import math
from typing import Any, Callable, Dict, NamedTuple, Optional

import torch

from moljax_gb300 import _native as N


class NKParams(NamedTuple):
    """newton_krylov.py:29-38 (+ gmres_restart; JAX's gmres default restart is 20)."""
    max_newton_iters: int = 10
    max_krylov_iters: int = 50
    newton_tol: float = 1e-8
    krylov_tol: float = 1e-6
    damping: float = 1.0
    backtrack_factor: float = 0.5
    max_backtrack: int = 3
    min_residual_decrease: float = 1e-4
    gmres_restart: int = 20


class NKStats(NamedTuple):
    converged: bool
    newton_iters: int
    lin_iters: int
    final_res_norm: float


class NKResult(NamedTuple):
    solution: Any
    stats: NKStats


def _cparams(p: NKParams) -> N.NKParamsC:
    return N.NKParamsC(p.max_newton_iters, p.max_krylov_iters, p.gmres_restart, p.max_backtrack,
                       p.newton_tol, p.krylov_tol, p.damping, p.backtrack_factor,
                       p.min_residual_decrease)


def integrate_implicit_vardiff(u0: torch.Tensor, dx: float, dt: float, n_steps: int,
                               method: str = "bdf2", a: float = 1.0, b: float = 1.0,
                               c: float = 1.0, nk_params: Optional[NKParams] = None,
                               be_guess: str = "euler", dy: Optional[float] = None):
    """Fixed-dt implicit steps on the GPU; u0 is an (n, n) interior (FP64 state).

    method: "be", "cn" or "bdf2" (BE first step, stepping.py:1077-1139).
    be_guess: "euler" (the explicit Euler guess of be_step/cn_step,
    stepping.py:195-196, 242-243) or "previous" (start Newton from y_n); BDF2
    steps always start from 2 y_n - y_{n-1} (stepping.py:299-300).  Returns (u, stats) where stats is an
    (n_steps, 3) int tensor of (Newton iterations, GMRES iterations, converged).
    """
    from moljax_gb300.core.fft_solvers import get_plan, workspace
    nk_params = nk_params or NKParams()
    u = u0.to(torch.float64).contiguous()
    N.require_cuda(u)
    n = u.shape[-1]
    dy = dx if dy is None else dy
    plan2 = get_plan(2 * n, 2 * n, dy, dx, "fd", torch.float32, u.device)
    lib = N.lib()
    ws = workspace(lib.mjx_nk_vardiff_ws_bytes(n, nk_params.gmres_restart), plan2.device, "nk")
    out = torch.empty_like(u)
    stats = (C.c_int * (3 * max(n_steps, 1)))()
    abc = (C.c_double * 3)(a, b, c)
    meth = {"be": 3, "cn": 4, "bdf2": 5}[method]
    cp = _cparams(nk_params)
    N.check("mjx_nk_vardiff_integrate2d", lib.mjx_nk_vardiff_integrate2d(
        N.ptr(plan2.buf), n, float(dy), float(dx), abc, meth, float(dt), int(n_steps),
        int(be_guess == "previous"), C.byref(cp), N.ptr(u), N.ptr(out), stats, N.ptr(ws),
        ws.numel(), N.stream_ptr(plan2.device)))
    st = torch.tensor(list(stats)[: 3 * n_steps], dtype=torch.int32).reshape(n_steps, 3)
    return out, st


# ----------------------------------------------------------------- generic form
def _flat(state):
    keys = list(state.keys())
    return torch.cat([state[k].reshape(-1) for k in keys]), keys, [state[k].shape for k in keys]


def _unflat(vec, keys, shapes):
    out, o = {}, 0
    for k, s in zip(keys, shapes):
        m = int(math.prod(s))
        out[k] = vec[o:o + m].reshape(s)
        o += m
    return out


def _gmres(matvec, b, tol, restart, maxiter, M=None):
    """Left-preconditioned restarted GMRES on flat torch vectors: classical Gram-Schmidt
    with one re-orthogonalisation pass, as jax.scipy.sparse.linalg.gmres orthogonalises
    (the Arnoldi basis is the rows of one device matrix, so a step is four matrix-vector
    products), Givens rotations and the small triangular solve on the host in FP64; one host
    synchronisation per Arnoldi step (its new Hessenberg column)."""
    import numpy as np
    Mf = M or (lambda v: v)
    bp = Mf(b)
    bnorm = float(torch.linalg.norm(bp))
    x = torch.zeros_like(b)
    its = 0
    if bnorm == 0.0:
        return x, 0
    for _ in range(maxiter):
        r = Mf(b - matvec(x)) if its else bp
        beta = float(torch.linalg.norm(r))
        if beta <= tol * bnorm:
            break
        V = torch.empty(restart + 1, b.numel(), dtype=b.dtype, device=b.device)
        V[0] = r / beta
        H = np.zeros((restart + 1, restart))
        cs, sn = np.zeros(restart), np.zeros(restart)
        g = np.zeros(restart + 1)
        g[0] = beta
        k = 0
        for j in range(restart):
            w = Mf(matvec(V[j]))
            Vj = V[:j + 1]
            h = Vj @ w
            w = w - Vj.T @ h
            h2 = Vj @ w
            w = w - Vj.T @ h2
            col = torch.cat([h + h2, torch.linalg.norm(w)[None]]).double().cpu().numpy()
            hn = float(col[j + 1])
            H[:j + 2, j] = col
            for i in range(j):
                t = cs[i] * H[i, j] + sn[i] * H[i + 1, j]
                H[i + 1, j] = -sn[i] * H[i, j] + cs[i] * H[i + 1, j]
                H[i, j] = t
            den = math.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = H[j, j] / den, H[j + 1, j] / den
            H[j, j], H[j + 1, j] = den, 0.0
            g[j + 1] = -sn[j] * g[j]
            g[j] = cs[j] * g[j]
            its += 1
            k = j + 1
            if abs(g[j + 1]) <= tol * bnorm or hn == 0.0:
                break
            V[j + 1] = w / hn
        y = np.zeros(k)
        for i in range(k - 1, -1, -1):  # back substitution (upper triangular)
            y[i] = (g[i] - H[i, i + 1:k] @ y[i + 1:k]) / H[i, i]
        x = x + V[:k].T @ torch.tensor(y, dtype=b.dtype, device=b.device)
        if abs(g[k]) <= tol * bnorm:
            break
    return x, its


def _native_solve(nat, x0, p: NKParams):
    """The solve of a create_implicit_residual / create_bdf2_residual residual over the
    variable-diffusion model on the native Newton-Krylov solver (mjx_nk_vardiff_step2d, guess
    x0): FP64 residual and Newton updates, FP32 JVP and GMRES, its DST preconditioner."""
    from moljax_gb300.core import stepping as S
    from moljax_gb300.core.fft_solvers import get_plan, workspace
    model = nat["model"]
    _, cp, abc, g = S._nk_setup(model, p)
    yn = S._interior64(model, nat["y_n"])
    yp = S._interior64(model, nat["y_prev"]) if nat["y_prev"] is not None else yn
    out = S._interior64(model, x0).clone()  # the guess, replaced by the root
    n = g.nx
    plan2 = get_plan(2 * n, 2 * n, g.dy, g.dx, "fd", torch.float32, yn.device)
    lib = N.lib()
    ws = workspace(lib.mjx_nk_vardiff_ws_bytes(n, p.gmres_restart), plan2.device, "nk")
    st = (C.c_int * 3)()
    rn = C.c_double(0.0)
    N.check("mjx_nk_vardiff_step2d", lib.mjx_nk_vardiff_step2d(
        N.ptr(plan2.buf), n, float(g.dy), float(g.dx), abc, int(nat["method"]), float(nat["dt"]),
        float(nat["dt_prev"]), 2, C.byref(cp), N.ptr(yn), N.ptr(yp), N.ptr(out), st, C.byref(rn), N.ptr(ws),
        ws.numel(), N.stream_ptr(plan2.device)))
    return NKResult({"u": S._padded(model, out, x0["u"])},
                    NKStats(bool(st[2]), int(st[0]), int(st[1]), float(rn.value)))


def newton_krylov_solve(residual_fn: Callable, x0, grid=None, params: Optional[Dict] = None,
                        preconditioner=None, nk_params: Optional[NKParams] = None, dt: float = 1.0,
                        *, gmres_restart: Optional[int] = None, rtol: Optional[float] = None):
    """Reference signature (newton_krylov.py:171-359) and README kwargs.

    ``rtol`` (README) sets newton_tol; ``gmres_restart`` sets the restart length.  A residual
    made by create_implicit_residual / create_bdf2_residual over the variable-diffusion model
    is solved by the native Newton-Krylov solver from x0 (its own preconditioner; the root is
    the same, GMRES counts differ); any other residual runs the torch form below (JVPs by
    torch.func, GMRES with one host synchronisation per Arnoldi step).
    """
    from moljax_gb300.core.preconditioners import PrecondContext, IdentityPreconditioner
    p = nk_params or NKParams()
    if rtol is not None:
        p = p._replace(newton_tol=rtol)
    if gmres_restart is not None:
        p = p._replace(gmres_restart=gmres_restart)
    nat = getattr(residual_fn, "native", None)
    if (nat is not None and isinstance(x0, dict) and set(x0) == {"u"}
            and "abc" in getattr(nat["model"], "metadata", {})):
        return _native_solve(nat, x0, p)
    single = not isinstance(x0, dict)
    x0d = {"x": x0} if single else x0
    res_fn = (lambda d: {"x": residual_fn(d["x"])}) if single else residual_fn
    xf, keys, shapes = _flat(x0d)
    ctx = PrecondContext(grid, dt, params or {})
    prec = preconditioner if preconditioner is not None else IdentityPreconditioner()

    def R(v):
        return _flat(res_fn(_unflat(v, keys, shapes)))[0]

    def M(v):
        return _flat(prec.apply(_unflat(v, keys, shapes), ctx))[0]

    use_m = not isinstance(prec, IdentityPreconditioner)
    x = xf.clone()
    rn = float(torch.linalg.norm(R(x)))
    converged = rn < p.newton_tol
    it = lits = 0
    res = rn
    while it < p.max_newton_iters and not converged:
        r = R(x)
        rn = float(torch.linalg.norm(r))
        converged = rn < p.newton_tol
        xc = x

        def jv(v):
            return torch.func.jvp(R, (xc,), (v,))[1]

        dx, li = _gmres(jv, -r, p.krylov_tol, p.gmres_restart, p.max_krylov_iters,
                        M if use_m else None)
        lits += li
        alpha, xb, rb, acc = p.damping, x, rn, False
        for _ in range(p.max_backtrack):
            if acc:
                break
            xn = xb + alpha * dx
            rnn = float(torch.linalg.norm(R(xn)))
            if rnn < (1.0 - p.min_residual_decrease * alpha) * rb:
                xb, rb, acc = xn, rnn, True
            else:
                alpha *= p.backtrack_factor
        x = xb if acc else x + p.damping * dx
        res = rb
        it += 1
    sol = _unflat(x, keys, shapes)
    return NKResult(sol["x"] if single else sol, NKStats(bool(converged), it, lits, res))


def create_implicit_residual(model, y_old, t_new: float, dt: float, method: str = "be"):
    """R(y) = y - y_old - dt F(y) ("be") or y - y_old - dt/2 (F(y_old) + F(y)) ("cn")
    (newton_krylov.py:362-403); F is the model's fused native rhs."""
    t_old = t_new - dt
    if method == "be":
        def residual(y_new):
            F = model.rhs(y_new, t_new)
            return {k: y_new[k] - y_old[k] - dt * F[k] for k in y_new}
    elif method == "cn":
        F_old = model.rhs(y_old, t_old)

        def residual(y_new):
            F = model.rhs(y_new, t_new)
            return {k: y_new[k] - y_old[k] - 0.5 * dt * (F_old[k] + F[k]) for k in y_new}
    else:
        raise ValueError(f"Unknown method: {method}")
    # what newton_krylov_solve needs to hand the solve to the native solver
    residual.native = {"model": model, "method": 3 if method == "be" else 4, "y_n": y_old, "y_prev": None,
                       "dt": dt, "dt_prev": dt}
    return residual


def create_bdf2_residual(model, y_n, y_nm1, t_new: float, dt: float, dt_prev: float):
    """Variable-step BDF2 residual a0 y + a1 y_n + a2 y_nm1 - beta F(y), omega = dt/dt_prev,
    a0 = (1+2w)/(1+w), a1 = -(1+w), a2 = w^2/(1+w), beta = dt (1+w)/(1+2w)
    (newton_krylov.py:406-448)."""
    w = dt / dt_prev
    a0, a1, a2 = (1.0 + 2.0 * w) / (1.0 + w), -(1.0 + w), w ** 2 / (1.0 + w)
    beta = dt * (1.0 + w) / (1.0 + 2.0 * w)

    def residual(y_new):
        F = model.rhs(y_new, t_new)
        return {k: a0 * y_new[k] + a1 * y_n[k] + a2 * y_nm1[k] - beta * F[k] for k in y_new}
    residual.native = {"model": model, "method": 5, "y_n": y_n, "y_prev": y_nm1, "dt": dt, "dt_prev": dt_prev}
    return residual
