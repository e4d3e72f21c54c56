"""Generic newton_krylov_solve (torch) on the reference's own NK test problems (CPU)."""

import numpy as np
import pytest
import torch


def test_nk_scalar_roots():
    # tests/test_nk.py:25-60: x^2 - 1 = 0 from 0.5 -> 1; 2x - 4 = 0 -> 2
    from moljax_gb300.core.newton_krylov import newton_krylov_solve
    r = newton_krylov_solve(lambda x: x * x - 1.0, torch.tensor([0.5], dtype=torch.float64))
    assert r.stats.converged and abs(float(r.solution[0]) - 1.0) < 1e-6
    r = newton_krylov_solve(lambda x: 2 * x - 4.0, torch.tensor([0.0], dtype=torch.float64))
    assert abs(float(r.solution[0]) - 2.0) < 1e-6 and r.stats.newton_iters <= 5


def test_nk_two_field_system():
    # tests/test_nk.py:62-97: coupled 2-field system
    from moljax_gb300.core.newton_krylov import newton_krylov_solve
    x0 = {"u": torch.tensor([0.5], dtype=torch.float64), "v": torch.tensor([0.5], dtype=torch.float64)}
    res = lambda s: {"u": s["u"] ** 2 + s["v"] ** 2 - 2.0, "v": s["u"] - s["v"]}  # noqa: E731
    r = newton_krylov_solve(res, x0)
    assert r.stats.converged
    assert abs(float(r.solution["u"][0]) - 1.0) < 1e-6 and abs(float(r.solution["v"][0]) - 1.0) < 1e-6


def test_nk_matches_oracle_newton():
    # same Newton/backtracking semantics as the oracle on a small nonlinear system
    from moljax_gb300.core.newton_krylov import newton_krylov_solve, NKParams
    from oracle import nk as ONK
    rng = np.random.default_rng(1)
    A = np.eye(6) * 4 + rng.standard_normal((6, 6)) * 0.3
    b = rng.standard_normal(6)
    resn = lambda x: A @ x + x ** 3 - b  # noqa: E731
    jvp = lambda x, v: A @ v + 3 * x * x * v  # noqa: E731
    xo, conv, it, li, rr = ONK.newton_krylov(resn, jvp, np.zeros(6), None, restart=20)
    At, bt = torch.tensor(A), torch.tensor(b)
    r = newton_krylov_solve(lambda x: At @ x + x ** 3 - bt, torch.zeros(6, dtype=torch.float64),
                            nk_params=NKParams())
    assert r.stats.newton_iters == it and r.stats.converged == bool(conv)
    np.testing.assert_allclose(r.solution.numpy(), xo, rtol=1e-10, atol=1e-12)


def test_nk_nonconvergence_reported():
    # tests/test_nk.py:190-229: max_newton_iters=1 with an impossible tolerance
    from moljax_gb300.core.newton_krylov import newton_krylov_solve, NKParams
    r = newton_krylov_solve(lambda x: x ** 3 - 2.0, torch.tensor([5.0], dtype=torch.float64),
                            nk_params=NKParams(max_newton_iters=1, newton_tol=1e-30))
    assert not r.stats.converged and r.stats.newton_iters == 1


def test_readme_kwargs_and_jacobi_preconditioner():
    # README.md:148-155 kwargs; reference DiffusionPreconditioner(field_diffusivities=...) form
    from moljax_gb300.core.newton_krylov import newton_krylov_solve
    from moljax_gb300.core.preconditioners import DiffusionPreconditioner
    p = DiffusionPreconditioner(field_diffusivities={"u": "D"})
    assert not p.spectral and p.n_iterations == 5 and p.omega == pytest.approx(0.6667)
    r = newton_krylov_solve(lambda x: x * x - 4.0, torch.tensor([1.0], dtype=torch.float64),
                            gmres_restart=30, rtol=1e-10)
    assert abs(float(r.solution[0]) - 2.0) < 1e-8


def test_oracle_controller_replay_matches_oracle_run():
    # the replayed controller (used to check the native adaptive implicit driver) makes the
    # same decisions as the oracle's own adaptive run
    from oracle import nk as ONK
    n = 16
    dx = 1.0 / n
    u0 = ONK.gaussians_ic(n)
    ro = ONK.adaptive_integrate_implicit(u0, dx, dx, "cn", 0.0, 0.01, 100 * dx * dx, atol=1e-4,
                                         rtol=1e-2, restart=20, be_guess="previous")
    rep = ONK.replay_implicit_controller(ro["log"], "cn", 0.0, 0.01, 100 * dx * dx)
    assert ro["status"] == 0 and len(rep) == len(ro["log"]) > 3
    for (t, dt, _, _, _, acc), (t2, dt2, acc2) in zip(ro["log"], rep):
        assert (t, dt, bool(acc)) == (t2, dt2, acc2)
