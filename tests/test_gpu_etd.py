"""ETD1, ETD2 and the library ETDRK4 on the GPU vs the NumPy FP64 oracle, and the
reference's own ETD test expectations (tests/test_fft_operators.py:393-617) run
through the native path."""

import numpy as np
import pytest
import torch

from oracle import etd as OT
from oracle import mol

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _grid1d(n):
    import moljax_gb300 as M
    g = M.Grid1D.uniform(n, x_min=0.0, x_max=1.0)
    return g, g.x_coords().numpy()


@pytest.mark.parametrize("method", ["etd1", "etd2", "etdrk4"])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_logistic_1d_vs_oracle(cuda, method, dtype):
    import moljax_gb300 as M
    n, D, alpha = 256, 0.01, 0.5
    g, x = _grid1d(n)
    u0 = 0.5 + 0.3 * np.sin(2 * np.pi * x)
    op = M.DiffusionOperator(g, D)
    t, hist = M.etd_integrate({"u": torch.tensor(u0, dtype=dtype, device=cuda)}, (0.0, 0.5), 0.05,
                              {"u": op}, M.NativeNonlinear.logistic(alpha), method=method, save_every=2)
    tr, hr = OT.etd_integrate({"u": u0}, (0.0, 0.5), 0.05, {"u": D * OT.fd_symbol_1d(n, g.dx)},
                              OT.logistic(alpha), method, 2)
    assert len(hist) == len(hr) == 6
    np.testing.assert_allclose(t.numpy(), tr, rtol=0, atol=1e-15)
    tol = 1e-12 if dtype == torch.float64 else 2e-6
    for a, b in zip(hist[1:], hr[1:]):
        assert _rel(a["u"].cpu().double().numpy(), b["u"]) < tol


@pytest.mark.parametrize("method", ["etd1", "etd2", "etdrk4"])
@pytest.mark.parametrize("n,dtype", [(32, torch.float64), (64, torch.float64), (64, torch.float32)])
def test_gray_scott_2d_vs_oracle(cuda, method, n, dtype):
    import moljax_gb300 as M
    L = 2.5
    grid = M.Grid2D(n, n, 0.0, L, 0.0, L)
    og = mol.Grid2D(n, n, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 11)
    u0, v0 = mol.interior(y0["u"], og), mol.interior(y0["v"], og)
    Du, Dv, F, k = 2e-5, 1e-5, 0.035, 0.065
    ops = {"u": M.DiffusionOperator(grid, Du), "v": M.DiffusionOperator(grid, Dv)}
    st = {"u": torch.tensor(u0, dtype=dtype, device=cuda), "v": torch.tensor(v0, dtype=dtype, device=cuda)}
    _, hist = M.etd_integrate(st, (0.0, 8.0), 1.0, ops, M.NativeNonlinear.gray_scott(F, k), method=method,
                              save_every=4)
    lam = mol.fd_symbol_2d(n, n, og.dy, og.dx)
    _, hr = OT.etd_integrate({"u": u0, "v": v0}, (0.0, 8.0), 1.0, {"u": Du * lam, "v": Dv * lam},
                             OT.gray_scott(F, k), method, 4, coupled=True)
    tol = 1e-11 if dtype == torch.float64 else 3e-6
    for f in ("u", "v"):
        assert _rel(hist[-1][f].cpu().double().numpy(), hr[-1][f]) < tol
        assert _rel(hist[1][f].cpu().double().numpy(), hr[1][f]) < tol


def test_etd2_step_chain_matches_integrate(cuda):
    import moljax_gb300 as M
    n = 128
    g, x = _grid1d(n)
    op = M.DiffusionOperator(g, 0.02)
    nl = M.NativeNonlinear.logistic(1.0)
    s = {"u": torch.tensor(0.5 + 0.3 * np.sin(2 * np.pi * x), device=cuda)}
    _, hist = M.etd_integrate(s, (0.0, 0.65), 0.1, {"u": op}, nl, method="etd2")  # int(0.65/0.1) = 6 steps
    Np = None
    st = s
    for i in range(6):
        st, Np = M.etd2_step(st, 0.1 * i, 0.1, {"u": op}, nl, Np)
        # etd2_step returns N at its input state
        if i == 0:
            assert _rel(Np["u"].cpu().numpy(), OT.logistic(1.0)({"u": s["u"].cpu().numpy()})["u"]) < 1e-14
    assert _rel(st["u"].cpu().numpy(), hist[-1]["u"].cpu().numpy()) < 1e-13
    # oracle chain
    so, Npo = {"u": s["u"].cpu().numpy()}, None
    for _ in range(6):
        so, Npo = OT.etd2_step(so, 0.1, {"u": 0.02 * OT.fd_symbol_1d(n, g.dx)}, OT.logistic(1.0), Npo)
    assert _rel(st["u"].cpu().numpy(), so["u"]) < 1e-12


def test_reference_etd_expectations(cuda):
    """tests/test_fft_operators.py:393-465 and 517-559 through the native path."""
    import moljax_gb300 as M
    zero = M.NativeNonlinear.zero()
    # ETD1 with N = 0 vs the pure exponential (< 1e-10)
    g, x = _grid1d(128)
    op = M.DiffusionOperator(g, 0.1)
    u0 = torch.tensor(np.sin(2 * np.pi * x), device=cuda)
    st = {"u": u0}
    for _ in range(10):
        st = M.etd1_step(st, 0.0, 0.01, {"u": op}, zero)
    pure = M.diffusion_only_etd1(u0, 0.1, 0.01, op)
    assert _rel(st["u"].cpu().numpy(), pure.cpu().numpy()) < 1e-10
    # etd_integrate API: 5 saves, within 1e-3 of the exact decay
    op = M.DiffusionOperator(g, 0.05)
    t, hist = M.etd_integrate({"u": u0}, (0.0, 0.2), 0.01, {"u": op}, zero, method="etd1", save_every=5)
    assert len(hist) == int(0.2 / 0.01 / 5) + 1
    exact = np.exp(-4 * np.pi ** 2 * 0.05 * 0.2) * np.sin(2 * np.pi * x)
    assert _rel(hist[-1]["u"].cpu().numpy(), exact) < 1e-3
    # ETDRK4 dt = 0.05 within 1 % of ETD1 dt = 0.001 (logistic, alpha = 0.1)
    g, x = _grid1d(256)
    op = M.DiffusionOperator(g, 0.01)
    u0 = {"u": torch.tensor(0.5 + 0.3 * np.sin(2 * np.pi * x), device=cuda)}
    nl = M.NativeNonlinear.logistic(0.1)
    a = M.etd_integrate(u0, (0.0, 1.0), 0.05, {"u": op}, nl, method="etdrk4")[1][-1]["u"].cpu().numpy()
    b = M.etd_integrate(u0, (0.0, 1.0), 0.001, {"u": op}, nl, method="etd1")[1][-1]["u"].cpu().numpy()
    assert np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)) < 0.01


def test_reference_etdrk4_order(cuda):
    """tests/test_fft_operators.py:561-617: observed ETDRK4 order > 3."""
    import moljax_gb300 as M
    g, x = _grid1d(256)
    op = M.DiffusionOperator(g, 0.01)
    nl = M.NativeNonlinear.logistic(0.5)
    u0 = {"u": torch.tensor(0.5 + 0.3 * np.sin(2 * np.pi * x), device=cuda)}
    ref = M.etd_integrate(u0, (0.0, 0.5), 0.0001, {"u": op}, nl, method="etdrk4")[1][-1]["u"].cpu().numpy()
    errs = [_rel(M.etd_integrate(u0, (0.0, 0.5), dt, {"u": op}, nl, method="etdrk4")[1][-1]["u"].cpu().numpy(),
                 ref) for dt in (0.1, 0.05, 0.025, 0.0125)]
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(3) if errs[i + 1] > 1e-14]
    assert np.mean(orders) > 3.0


def test_field_without_operator_is_explicit(cuda):
    # no linear operator: ETD1 = explicit Euler (fft_integrators.py:172-174)
    import moljax_gb300 as M
    g, x = _grid1d(64)
    u0 = 0.5 + 0.3 * np.sin(2 * np.pi * x)
    st = M.etd1_step({"u": torch.tensor(u0, device=cuda)}, 0.0, 0.1, {}, M.NativeNonlinear.logistic(2.0))
    ref = OT.etd1_step({"u": u0}, 0.1, {}, OT.logistic(2.0))
    assert _rel(st["u"].cpu().numpy(), ref["u"]) < 1e-14


def test_native_nonlinear_and_1d_operator(cuda):
    import moljax_gb300 as M
    n = 128
    g, x = _grid1d(n)
    u = 0.5 + 0.3 * np.sin(2 * np.pi * x) + 0.1 * np.cos(6 * np.pi * x)
    ut = torch.tensor(u, device=cuda)
    out = M.NativeNonlinear.logistic(0.7)({"u": ut})["u"].cpu().numpy()
    np.testing.assert_allclose(out, 0.7 * u * (1 - u), rtol=1e-14, atol=1e-15)
    gsn = M.NativeNonlinear.gray_scott(0.035, 0.065)({"u": ut, "v": ut * 0.5})
    ref = OT.gray_scott(0.035, 0.065)({"u": u, "v": 0.5 * u})
    for f in ("u", "v"):
        np.testing.assert_allclose(gsn[f].cpu().numpy(), ref[f], rtol=1e-13, atol=1e-15)
    op = M.DiffusionOperator(g, 0.03)
    lam = 0.03 * OT.fd_symbol_1d(n, g.dx)
    uh = np.fft.fft(u)
    np.testing.assert_allclose(op.matvec(ut).cpu().numpy(), np.real(np.fft.ifft(lam * uh)), rtol=0, atol=1e-11)
    np.testing.assert_allclose(op.solve(ut, 0.2).cpu().numpy(), np.real(np.fft.ifft(uh / (1 - 0.2 * lam))),
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(op.exp_matvec(ut, 0.2).cpu().numpy(), np.real(np.fft.ifft(np.exp(0.2 * lam) * uh)),
                               rtol=0, atol=1e-13)
    np.testing.assert_allclose(op.eigenvalues.numpy(), lam, rtol=1e-14)


@pytest.mark.parametrize("method", ["etdrk4", "etd1"])
def test_adaptive_etd_1d_vs_oracle(cuda, method):
    import moljax_gb300 as M
    from oracle import imex as OI
    n = 128
    g, x = _grid1d(n)
    u0 = 0.5 + 0.3 * np.sin(2 * np.pi * x)
    op = M.DiffusionOperator(g, 0.01)
    rtol, atol = (1e-7, 1e-9) if method == "etdrk4" else (1e-4, 1e-6)
    pid = M.PIDParams(rtol=rtol, atol=atol)
    r = M.etd_adaptive_integrate({"u": torch.tensor(u0, device=cuda)}, 0.0, 2.0, 0.05, {"u": op},
                                 M.NativeNonlinear.logistic(2.0), method=method, pid_params=pid)
    o = OT.adaptive_etd({"u": u0}, 0.0, 2.0, 0.05, {"u": 0.01 * OT.fd_symbol_1d(n, g.dx)}, OT.logistic(2.0),
                        method, OI.PIDParams(rtol=rtol, atol=atol))
    assert (r.status, r.n_accepted, r.n_rejected) == (o.status, o.n_accepted, o.n_rejected)
    assert r.status == 0 and r.n_accepted > 3
    # the step-doubling estimate divides an O(rtol |u|) difference of two solutions by
    # rtol |u|, so the ~1e-15 rounding of each solution's transforms (Stockham on the GPU,
    # pocketfft in the oracle) reaches the error ratio as ~1e-15 / rtol and the dt
    # sequence through the PI controller: rtol 1e-7 -> ~1e-7 relative in dt
    np.testing.assert_allclose(r.t_history.numpy()[:r.n_steps], o.t_history[:o.n_steps], rtol=1e-5)
    assert _rel(r.y_final["u"].cpu().numpy(), o.y_final["u"]) < 1e-9


def test_adaptive_etdrk4_gray_scott_vs_oracle(cuda):
    import moljax_gb300 as M
    from oracle import imex as OI
    n, L = 32, 2.5
    grid = M.Grid2D(n, n, 0.0, L, 0.0, L)
    og = mol.Grid2D(n, n, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 5)
    u0, v0 = mol.interior(y0["u"], og), mol.interior(y0["v"], og)
    Du, Dv, F, k = 2e-5, 1e-5, 0.035, 0.065
    ops = {"u": M.DiffusionOperator(grid, Du), "v": M.DiffusionOperator(grid, Dv)}
    st = {"u": torch.tensor(u0, device=cuda), "v": torch.tensor(v0, device=cuda)}
    pid = dict(rtol=1e-6, atol=1e-8, dt_max=20.0)
    r = M.etd_adaptive_integrate(st, 0.0, 200.0, 1.0, ops, M.NativeNonlinear.gray_scott(F, k),
                                 pid_params=M.PIDParams(**pid))
    lam = mol.fd_symbol_2d(n, n, og.dy, og.dx)
    o = OT.adaptive_etd({"u": u0, "v": v0}, 0.0, 200.0, 1.0, {"u": Du * lam, "v": Dv * lam}, OT.gray_scott(F, k),
                        "etdrk4", OI.PIDParams(**pid), coupled=True)
    assert (r.status, r.n_accepted, r.n_rejected) == (o.status, o.n_accepted, o.n_rejected)
    # v decays to ~1e-12 by t = 200 here, so compare on the O(1) scale of the fields
    for f in ("u", "v"):
        assert float(np.max(np.abs(r.y_final[f].cpu().numpy() - o.y_final[f]))) < 1e-9
