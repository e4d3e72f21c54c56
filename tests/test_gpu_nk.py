"""Native Newton-Krylov implicit steps vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import nk as ONK

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("method", ["bdf2", "be", "cn"])
def test_nk_steps_vs_oracle(cuda, method):
    import moljax_gb300 as M
    n = 64
    dx = 1.0 / n
    u0 = ONK.gaussians_ic(n)
    dt = 100 * dx * dx
    nkp = M.NKParams(gmres_restart=30)
    u, st = M.integrate_implicit_vardiff(torch.tensor(u0, device=cuda), dx, dt, 4, method=method,
                                         nk_params=nkp, be_guess="previous")
    ref, rst = _oracle(u0, dx, dt, 4, method)
    assert _rel(u.cpu().numpy(), ref) < 1e-7
    assert bool(st[:, 2].all())
    # Newton iteration counts: same up to one (FP32 Krylov vs FP64 oracle)
    assert np.max(np.abs(st[:, 0].numpy() - np.array([s[0] for s in rst]))) <= 1


def _oracle(u0, dx, dt, n, method):
    if method == "bdf2":
        return ONK.bdf2_integrate(u0, dx, dx, dt, n, restart=30, be_guess="previous")
    F = lambda u: ONK.vardiff_F(u, dx, dx)  # noqa: E731
    J = lambda u, v: ONK.vardiff_JF(u, v, dx, dx)  # noqa: E731
    u = u0.copy()
    stats = []
    for _ in range(n):
        if method == "be":
            a0, beta, cst, guess = 1.0, dt, -u, u.copy()
        else:
            a0, beta, cst, guess = 1.0, 0.5 * dt, -u - 0.5 * dt * F(u), u.copy()
        Db = 1.0 + float(np.mean(u * u))
        res = lambda y: a0 * y + cst - beta * F(y)  # noqa: E731
        jvp = lambda y, v: a0 * v - beta * J(y, v)  # noqa: E731
        Mi = lambda r: ONK.dirichlet_helmholtz(r, dx, dx, a0, beta * Db)  # noqa: E731
        u, conv, it, li, rr = ONK.newton_krylov(res, jvp, guess, Mi, restart=30)
        stats.append((it, li, conv))
    return u, stats


def test_dirichlet_preconditioner_vs_oracle(cuda):
    from moljax_gb300.core.preconditioners import dirichlet_helmholtz
    rng = np.random.default_rng(3)
    r = rng.standard_normal((32, 32))
    out = dirichlet_helmholtz(torch.tensor(r, device=cuda), 0.1, 0.1, 1.5, 0.02).cpu().numpy()
    ref = ONK.dirichlet_helmholtz(r, 0.1, 0.1, 1.5, 0.02)
    assert _rel(out, ref) < 1e-12


def test_nk_reports_nonconvergence(cuda):
    # impossible tolerance: every step reports converged = 0 after max_newton_iters
    import moljax_gb300 as M
    n = 32
    dx = 1.0 / n
    u0 = ONK.gaussians_ic(n)
    nkp = M.NKParams(newton_tol=1e-30, max_newton_iters=2, gmres_restart=10)
    u, st = M.integrate_implicit_vardiff(torch.tensor(u0, device=cuda), dx, 100 * dx * dx, 2,
                                         nk_params=nkp, be_guess="previous")
    assert not bool(st[:, 2].any())
    assert (st[:, 0] == 2).all()


def _vardiff_setup(n, cuda):
    import moljax_gb300 as M
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_variable_diffusion_model(grid)
    u0 = ONK.gaussians_ic(n)
    y = torch.zeros((n + 2, n + 2), dtype=torch.float64, device=cuda)
    y[1:-1, 1:-1] = torch.tensor(u0, device=cuda)
    y = model.apply_bcs({"u": y})
    return M, grid, model, u0, y


def test_vardiff_rhs_vs_oracle(cuda):
    M, grid, model, u0, y = _vardiff_setup(32, cuda)
    F = model.rhs(y)["u"].cpu().numpy()
    ref = ONK.vardiff_F(u0, grid.dy, grid.dx)
    assert _rel(F[1:-1, 1:-1], ref) < 1e-13
    assert np.all(F[0, :] == 0) and np.all(F[:, -1] == 0)  # ghosts zeroed


@pytest.mark.parametrize("method", ["be", "cn", "bdf2"])
def test_single_implicit_steps_vs_oracle(cuda, method):
    # be_step / cn_step / bdf2_step (variable step: dt != dt_prev) against the oracle
    M, grid, model, u0, y = _vardiff_setup(32, cuda)
    dx = grid.dx
    dt, dt_prev = 60 * dx * dx, 100 * dx * dx
    nkp = M.NKParams(gmres_restart=30)
    u_prev0 = 0.9 * u0
    # the explicit-Euler guess of be_step/cn_step diverges at this stiff dt: start from y_n
    if method == "be":
        out, st = M.be_step(model, y, 0.0, dt, nk_params=nkp, be_guess="previous")
    elif method == "cn":
        out, st = M.cn_step(model, y, 0.0, dt, nk_params=nkp, be_guess="previous")
    else:
        yp = {"u": y["u"] * 0.9}
        out, st = M.bdf2_step(model, y, yp, 0.0, dt, dt_prev, nk_params=nkp)
    ref, conv, it, _ = ONK.implicit_step(u0, u_prev0, method, dt, dt_prev, dx, dx, restart=30,
                                         be_guess="previous")
    assert st.converged and conv
    assert abs(st.newton_iters - it) <= 1
    assert _rel(out["u"][1:-1, 1:-1].cpu().numpy(), ref) < 1e-7
    g = out["u"].cpu().numpy()
    np.testing.assert_array_equal(g[0, 1:-1], -g[1, 1:-1])  # Dirichlet ghosts refilled


@pytest.mark.parametrize("method", ["be", "cn"])
def test_euler_guess_steps_vs_oracle(cuda, method):
    # the reference's explicit-Euler initial guess, at a dt where explicit Euler is stable
    M, grid, model, u0, y = _vardiff_setup(32, cuda)
    dt = 0.1 * grid.dx ** 2
    step = M.be_step if method == "be" else M.cn_step
    out, st = step(model, y, 0.0, dt, nk_params=M.NKParams(gmres_restart=30))
    ref, conv, it, _ = ONK.implicit_step(u0, u0, method, dt, dt, grid.dx, grid.dx, restart=30)
    assert st.converged and conv and abs(st.newton_iters - it) <= 1
    assert _rel(out["u"][1:-1, 1:-1].cpu().numpy(), ref) < 1e-9


def test_integrate_fixed_dt_matches_fused_path(cuda):
    M, grid, model, u0, y = _vardiff_setup(32, cuda)
    dt = 100 * grid.dx ** 2
    nkp = M.NKParams(gmres_restart=30)
    t, ys, yf = M.integrate_fixed_dt(model, y, 0.0, 3.5 * dt, dt, M.IntegratorType.BDF2,
                                     nk_params=nkp, be_guess="previous")
    assert t.numel() == 4 and ys["u"].shape == (4, 34, 34)
    u, _ = M.integrate_implicit_vardiff(torch.tensor(u0, device=cuda), grid.dx, dt, 4,
                                        method="bdf2", nk_params=nkp, be_guess="previous")
    assert _rel(yf["u"][1:-1, 1:-1].cpu().numpy(), u.cpu().numpy()) < 1e-13


@pytest.mark.parametrize("method", ["be", "cn", "bdf2"])
def test_adaptive_implicit_vs_oracle(cuda, method):
    # implicit branch of adaptive_integrate: error vs a BE solve (BE: dt F), PI + robustness dt.
    # The dt sequence feeds on Newton iteration counts (<= 3 grows dt by 1.2), which FP32
    # Krylov vectors can shift by one against the FP64 oracle, so the controller is checked by
    # replaying it on the recorded attempts, and the trajectory against the oracle's own run
    # within the integration tolerance.
    M, grid, model, u0, y = _vardiff_setup(32, cuda)
    dx = grid.dx
    itype = {"be": M.IntegratorType.BE, "cn": M.IntegratorType.CN, "bdf2": M.IntegratorType.BDF2}
    pid = M.PIDParams(atol=1e-4, rtol=1e-2)
    log = []
    dt0 = 100 * dx * dx
    r = M.adaptive_integrate(model, y, 0.0, 0.005, dt0, itype[method], max_steps=2000,
                             pid_params=pid, nk_params=M.NKParams(gmres_restart=30),
                             be_guess="previous", attempt_log=log)
    assert r.status == 0 and r.t_final == pytest.approx(0.005, rel=1e-12)
    assert len(log) == r.n_accepted + r.n_rejected
    assert sum(a[5] for a in log) == r.n_accepted
    want = ONK.replay_implicit_controller(log, method, 0.0, 0.005, dt0)
    for got, exp in zip(log, want):
        assert got[0] == pytest.approx(exp[0], rel=1e-12, abs=1e-15)
        assert got[1] == pytest.approx(exp[1], rel=1e-12)
        assert bool(got[5]) == exp[2]
    k = r.n_steps
    np.testing.assert_allclose(r.t_history.numpy()[:k],
                               np.concatenate([[0.0], np.cumsum([a[1] for a in log if a[5]])])[:k],
                               rtol=1e-12)
    ro = ONK.adaptive_integrate_implicit(u0, dx, dx, method, 0.0, 0.005, dt0, atol=1e-4,
                                         rtol=1e-2, max_steps=2000, restart=30,
                                         be_guess="previous")
    assert ro["status"] == 0
    assert abs(r.n_accepted - ro["n_acc"]) <= 0.25 * ro["n_acc"] + 2
    # both runs meet rtol = 1e-2 per step; their final states agree far inside that
    assert _rel(r.y_final["u"][1:-1, 1:-1].cpu().numpy(), ro["u"]) < 5e-3


def test_vardiff_jvp_vs_oracle_and_difference_quotient(cuda):
    """The exported hand-written JVP equals the oracle's JVP and the central difference
    of the native F (jax.jvp's role in newton_krylov.py:61-80)."""
    import moljax_gb300 as M
    from moljax_gb300.core.model import vardiff_jvp
    n = 48
    g = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    m = M.create_variable_diffusion_model(g, 1.0, 1.0, 1.0)
    rng = np.random.default_rng(9)
    u = ONK.gaussians_ic(n)
    v = rng.standard_normal((n, n))
    ut, vt = torch.tensor(u, device=cuda), torch.tensor(v, device=cuda)
    jv = vardiff_jvp(m, ut, vt).cpu().numpy()
    ref = ONK.vardiff_JF(u, v, 1.0 / n, 1.0 / n)
    assert _rel(jv, ref) < 1e-13
    # the residual form a0 v - beta J v
    jr = vardiff_jvp(m, ut, vt, a0=1.5, beta=0.01).cpu().numpy()
    assert _rel(jr, 1.5 * v - 0.01 * ref) < 1e-13
    eps = 1e-6
    Fp = ONK.vardiff_F(u + eps * v, 1.0 / n, 1.0 / n)
    Fm = ONK.vardiff_F(u - eps * v, 1.0 / n, 1.0 / n)
    assert _rel(jv, (Fp - Fm) / (2 * eps)) < 1e-7


@pytest.mark.parametrize("method", ["be", "cn", "bdf2"])
def test_newton_krylov_solve_routes_factory_residuals(cuda, method):
    """newton_krylov_solve on a create_implicit_residual / create_bdf2_residual residual of
    the variable-diffusion model runs the native solver from the given guess: the same root as
    be_step / cn_step / bdf2_step and the oracle."""
    import moljax_gb300 as M
    M_, grid, model, u0, y = _vardiff_setup(32, cuda)
    dx = grid.dx
    dt, dt_prev = 60 * dx * dx, 100 * dx * dx
    nkp = M.NKParams(gmres_restart=30)
    yp = {"u": y["u"] * 0.9}
    if method == "bdf2":
        res = M.create_bdf2_residual(model, y, yp, dt, dt, dt_prev)
        ref, conv, it, _ = ONK.implicit_step(u0, 0.9 * u0, method, dt, dt_prev, dx, dx, restart=30)
        guess = {"u": 2 * y["u"] - yp["u"]}
    else:
        res = M.create_implicit_residual(model, y, dt, dt, method)
        ref, conv, it, _ = ONK.implicit_step(u0, u0, method, dt, dt, dx, dx, restart=30, be_guess="previous")
        guess = {"u": y["u"].clone()}
    assert hasattr(res, "native")
    out = M.newton_krylov_solve(res, guess, nk_params=nkp)
    assert out.stats.converged and conv and abs(out.stats.newton_iters - it) <= 1
    assert _rel(out.solution["u"][1:-1, 1:-1].cpu().numpy(), ref) < 1e-7


def test_generic_gmres_entry(cuda):
    """mjx_gmres_solve with host callbacks that enqueue library kernels: A = (I - h D Lap)^-1
    (a periodic Helmholtz solve, condition number ~34 here), without a preconditioner and with
    the mild SPD left preconditioner (I - h' D Lap)^-1, h' = h/100; the solution must be
    (I - h D Lap) b.  A callback that reports failure aborts the solve."""
    import ctypes as C
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import get_plan
    n = 64
    plan = get_plan(n, n, 1.0 / n, 1.0 / n, "fd", torch.float32, cuda)
    lib = N.lib()
    wsz = plan.ws_bytes(1)
    wsp = torch.empty(wsz, dtype=torch.uint8, device=cuda)
    h, D = 1e-3, 1.0
    Dc = (C.c_double * 1)(D)

    def op(mult, hh):
        def f(v, out, user, stream):
            return lib.mjx_spectral_apply2d(N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, 1, Dc, hh, mult, v, out,
                                            N.ptr(wsp), wsz, stream)
        return N.VecOp(f)
    A, P = op(N.MULT_HELMHOLTZ, h), op(N.MULT_HELMHOLTZ, 0.01 * h)
    rng = np.random.default_rng(2)
    b = torch.tensor(rng.standard_normal((n, n)), dtype=torch.float32, device=cuda)
    exact = b - plan.apply(b, D, h, N.MULT_LAP)  # (I - h D Lap) b
    gw = torch.empty(lib.mjx_gmres_ws_bytes(n * n, 30), dtype=torch.uint8, device=cuda)
    stream = N.stream_ptr(cuda)
    for pre in (N.VecOp(), P):  # VecOp(): a NULL callback, no preconditioner
        x = torch.zeros_like(b)
        its, conv, rr = C.c_int(), C.c_int(), C.c_double()
        N.check("mjx_gmres_solve", lib.mjx_gmres_solve(n * n, A, pre, None, N.ptr(b), N.ptr(x), 1e-5, 30, 20,
                                                      C.byref(its), C.byref(rr), C.byref(conv), N.ptr(gw),
                                                      gw.numel(), stream))
        assert conv.value == 1 and 0 < its.value <= 600 and rr.value <= 1e-5, (its.value, rr.value)
        assert float(torch.linalg.norm(x - exact) / torch.linalg.norm(exact)) < 1e-3
    bad = N.VecOp(lambda v, out, user, stream: 1)
    assert lib.mjx_gmres_solve(n * n, bad, N.VecOp(), None, N.ptr(b), N.ptr(x), 1e-5, 30, 10, C.byref(its),
                               C.byref(rr), C.byref(conv), N.ptr(gw), gw.numel(), stream) != 0


_NK_HOST_CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np, torch
import moljax_gb300 as M
from oracle import nk as ONK
n = 64
u0 = ONK.gaussians_ic(n)
dx = 1.0 / n
u, st = M.integrate_implicit_vardiff(torch.tensor(u0, device="cuda"), dx, 100 * dx * dx, 4, method="bdf2",
                                     nk_params=M.NKParams(gmres_restart=30), be_guess="previous")
np.savez(sys.argv[2], u=u.cpu().numpy(), st=st.cpu().numpy())
"""


def test_device_newton_loop_matches_host_loop(cuda, tmp_path):
    """The Newton iteration as one graph of nested conditional loops (default) against the
    host-driven iteration (MJX_HOST_LOOP=1, read once per process): the same kernels and the
    same decisions, so the same Newton / GMRES counts and the same states."""
    import os
    import subprocess
    import sys
    import moljax_gb300 as M
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = str(tmp_path / "nk_host.npz")
    subprocess.run([sys.executable, "-c", _NK_HOST_CHILD, root, path], env=dict(os.environ, MJX_HOST_LOOP="1"),
                   check=True, timeout=600)
    child = np.load(path)
    n = 64
    u0 = ONK.gaussians_ic(n)
    dx = 1.0 / n
    u, st = M.integrate_implicit_vardiff(torch.tensor(u0, device=cuda), dx, 100 * dx * dx, 4, method="bdf2",
                                         nk_params=M.NKParams(gmres_restart=30), be_guess="previous")
    np.testing.assert_array_equal(st.cpu().numpy(), child["st"])
    assert _rel(u.cpu().numpy(), child["u"]) < 1e-12
