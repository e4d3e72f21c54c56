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
