"""The oracle against the reference's published numbers and known answers (CPU)."""

import json
import os

import numpy as np
import pytest

from oracle import fftcn, imex, mol

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    with open(os.path.join(GOLD, name)) as f:
        return json.load(f)


@pytest.mark.parametrize("row", _load("fftcn_published.json")["precision_table"]["fp64"])
def test_fftcn_error_table_fp64(row):
    # benchmarks/results/precision_fp32_fp64.json: 128^2, D=0.1, T=0.1, max error vs analytic
    g = _load("fftcn_published.json")
    D, T = g["precision_table"]["D"], g["precision_table"]["t_final"]
    u0 = fftcn.node_grid_ic(128)
    n = int(T / row["dt"])
    assert n == row["n_steps"]
    u = fftcn.fft_cn_2d(u0, D, 1.0 / 128, row["dt"], n)
    err = np.max(np.abs(u - fftcn.analytic_decay(u0, D, n * row["dt"])))
    # the published value carries FP64 rounding of the reference run (~1e-16 * steps)
    assert err == pytest.approx(row["error"], rel=1e-9, abs=2e-14 * n)


def test_fftcn_scipy_comparison_bitwise():
    # benchmarks/results/scipy_comparison.json: the NumPy FFT-CN error, reproduced exactly
    s = _load("fftcn_published.json")["scipy_comparison"]
    u0 = fftcn.node_grid_ic(128)
    u = fftcn.fft_cn_2d(u0, s["D"], 1.0 / 128, s["dt"], s["n_steps"])
    err = np.max(np.abs(u - fftcn.analytic_decay(u0, s["D"], s["t_final"])))
    assert err == pytest.approx(s["numpy_error"], rel=1e-12)
    assert err == pytest.approx(s["jax_error"], rel=1e-5)


def test_fd_symbol_zero_mode_and_sign():
    # tests/test_fft_solver.py:43-57
    lam = mol.fd_symbol_2d(16, 16, 0.1, 0.1)
    assert lam[0, 0] == pytest.approx(0.0, abs=1e-12)
    assert np.all(lam.ravel()[1:] < 0)


def test_helmholtz_residual():
    # tests/test_fft_solver.py:140-205: (I - dt D lam) u = rhs in Fourier space
    rng = np.random.default_rng(0)
    rhs = rng.standard_normal((32, 32))
    lam = mol.fd_symbol_2d(32, 32, 1 / 32, 1 / 32)
    u = mol.solve_helmholtz_2d(rhs, lam, 0.01, 0.1)
    back = np.fft.ifft2(np.fft.fft2(u) * (1 - 0.01 * 0.1 * lam)).real
    assert np.max(np.abs(back - rhs)) < 1e-12


def test_helmholtz_fd_residual():
    # tests/test_fft_solver.py:207-247: u - dt D Lap_FD(u) == rhs with periodic ghosts
    g = mol.Grid2D(32, 32, 0, 1, 0, 1)
    rng = np.random.default_rng(1)
    rhs = rng.standard_normal((32, 32))
    lam = mol.fd_symbol_2d(32, 32, g.dy, g.dx)
    u = mol.solve_helmholtz_2d(rhs, lam, 0.01, 0.1)
    up = mol.bc_2d(mol.pad(u, g), g, mol.PERIODIC)
    lap = mol.interior(mol.laplacian_2d(up, g), g)
    assert np.max(np.abs(u - 0.01 * 0.1 * lap - rhs)) < 1e-10


def _gs(n=32):
    g = mol.Grid2D(n, n, 0, 2.5, 0, 2.5)
    model, lam, diff = imex.gray_scott_periodic(g, 2e-5, 1e-5, 0.035, 0.065)
    return g, model, lam, diff


def test_imex_pure_diffusion_decay():
    # tests/test_imex.py:99-136: sin mode decays like exp(-2 D t) (rtol 0.01)
    n = 32
    g = mol.Grid2D(n, n, 0, 2 * np.pi, 0, 2 * np.pi)
    model = imex.Model(g, {"u": mol.PERIODIC}, {}, None)
    lam = mol.fd_symbol_2d(n, n, g.dy, g.dx)
    X, Y = g.meshgrid(include_ghost=True)
    y = {"u": np.sin(X) * np.sin(Y)}
    D, dt = 0.1, 0.01
    for _ in range(100):
        y = imex.imex_strang_step(model, y, dt, lam, {"u": D})
    ratio = np.max(np.abs(mol.interior(y["u"], g))) / np.max(np.abs(np.sin(X) * np.sin(Y))[g.interior_slice])
    assert ratio == pytest.approx(np.exp(-2 * D * 1.0), rel=0.01)


def test_fixed_dt_equals_manual_steps():
    # tests/test_imex.py:233-259
    g, model, lam, diff = _gs(16)
    y0 = mol.gray_scott_ic(g, seed=3)
    ts, ys, yf = imex.integrate_imex_fixed_dt(model, y0, 0.0, 2.0, 0.5, lam, diff)
    y = y0
    for _ in range(len(ts)):
        y = imex.imex_strang_step(model, y, 0.5, lam, diff)
    for k in y:
        assert np.max(np.abs(y[k] - yf[k])) < 1e-10


def test_adaptive_imex_success_and_accept_rate():
    # tests/test_imex.py:185-231: SUCCESS, accept rate > 0.5, bounded GS fields
    g, model, lam, diff = _gs(16)
    y0 = mol.gray_scott_ic(g, seed=4)
    pid = imex.PIDParams(atol=1e-7, rtol=1e-5)
    r = imex.adaptive_integrate_imex(model, y0, 0.0, 20.0, 1.0, lam, diff, pid=pid,
                                     save_every=100, keep_history=False)
    assert r.status == imex.SUCCESS
    assert r.t_final == pytest.approx(20.0)
    assert r.n_accepted / (r.n_accepted + r.n_rejected) > 0.5
    for k in r.y_final:
        assert np.all(np.isfinite(r.y_final[k]))
        assert np.all(r.y_final[k] > -0.5) and np.all(r.y_final[k] < 1.5)


def test_controller_formulas():
    # dt_policy.py:178-268 by hand
    pid = imex.PIDParams()
    dt, pe = imex.pid_controller_dt(0.1, 0.5, 1.0, pid, 2)
    fac = min(max((2.0 ** 0.35) * ((1.0 / 0.5) ** 0.2) * 0.9, 0.2), 5.0)
    assert dt == pytest.approx(0.1 * fac) and pe == 0.5
    assert imex.handle_rejected_step(0.1, 4.0, pid, 2) == pytest.approx(0.1 * 0.9 * 0.25 ** 0.35)
    assert imex.handle_rejected_step(0.1, 1e6, pid, 2) == pytest.approx(0.02)


def test_imex_cfl_gray_scott():
    # dt_policy.py:430-502: reaction limit 0.5/(F+k) -> 5, capped by dt_max 1, x safety 0.9
    g = mol.Grid2D(8, 8, 0, 1, 0, 1)
    assert imex.imex_cfl_dt(g, {"F": 0.035, "k": 0.065}, imex.CFLParams()) == pytest.approx(0.9)


def test_bc_formulas_2d():
    # tests/test_bc.py: periodic wrap, Dirichlet 2b-u, Neumann u -/+ 2 dx q
    g = mol.Grid2D(4, 3, 0, 1, 0, 1)
    rng = np.random.default_rng(2)
    f = rng.standard_normal((5, 6))
    p = mol.bc_2d(f, g, mol.PERIODIC)
    assert np.allclose(p[1:-1, 0], f[1:-1, 4]) and np.allclose(p[0, 1:-1], p[3, 1:-1])
    d = mol.bc_2d(f, g, mol.DIRICHLET, {"left": 1.0})
    assert np.allclose(d[1:-1, 0], 2.0 - f[1:-1, 1])
    n = mol.bc_2d(f, g, mol.NEUMANN, {"top": 0.5})
    assert np.allclose(n[4, :], n[3, :] + 2 * g.dy * 0.5)


def test_etdrk4_oracle_orders():
    # Cox-Matthews form is 4th order (tests/test_fft_operators.py:561-617: order > 3);
    # the benchmark-script form (f2 without the factor 2) is not
    from oracle import etdrk4 as OE
    n, L = 16, 2.5
    g = mol.Grid2D(n, n, 0, L, 0, L)
    y0 = mol.gray_scott_ic(g, 3)
    u0, v0 = mol.interior(y0["u"], g), mol.interior(y0["v"], g)
    lam = mol.fd_symbol_2d(n, n, g.dy, g.dx)
    args = (u0, v0, lam, 2e-3, 1e-3, 0.035, 0.065)
    for fac, lo in ((2.0, 12.0), (1.0, None)):
        ref = OE.etdrk4_gray_scott(*args, 0.0625, 128, fac)[0]
        e1 = np.linalg.norm(OE.etdrk4_gray_scott(*args, 2.0, 4, fac)[0] - ref)
        e2 = np.linalg.norm(OE.etdrk4_gray_scott(*args, 1.0, 8, fac)[0] - ref)
        if lo is not None:
            assert e1 / e2 > lo
        else:
            assert e1 / e2 < 4.0


# ---------------------------------------------------------------- DST-I (fft_nonperiodic.py)
def test_dst_oracle_pins():
    import scipy.fft
    from oracle import dst as OD
    # tests/test_fft_nonperiodic.py:24-33: DST then IDST recovers the input (rtol 1e-10)
    N = 32
    x = np.sin(np.pi * np.arange(1, N + 1) / (N + 1))
    np.testing.assert_allclose(OD.idst_I_fast(OD.dst_I_fast(x)), x, rtol=1e-10)
    # 35-46: DST of sin(pi x) concentrates in mode 1
    N = 64
    f = np.sin(np.pi * np.arange(1, N + 1) / (N + 1))
    F = OD.dst_I_fast(f)
    assert abs(F[0]) > 0.9 * np.linalg.norm(F)
    # eigenvalues negative and increasing in magnitude (52-70)
    lam = OD.laplacian_symbol_dirichlet(32, 0.1)
    assert np.all(lam < 0) and np.all(np.diff(np.abs(lam)) >= 0)
    # scipy's type-1 DST is twice this transform, for any N
    rng = np.random.default_rng(0)
    for N in (1, 2, 7, 33, 100):
        x = rng.standard_normal((3, N))
        np.testing.assert_allclose(OD.dst_I_fast(x), 0.5 * scipy.fft.dst(x, type=1, axis=-1),
                                   rtol=1e-12, atol=1e-12)
    # the Helmholtz solve inverts (I - dt D Lap_D) with the 3-point Dirichlet Laplacian
    N, dx, dt, D = 50, 0.02, 0.3, 0.7
    u = rng.standard_normal(N)
    lam = OD.laplacian_symbol_dirichlet(N, dx)
    A = (np.diag(-2.0 * np.ones(N)) + np.diag(np.ones(N - 1), 1) + np.diag(np.ones(N - 1), -1)) / dx ** 2
    rhs = u - dt * D * A @ u
    np.testing.assert_allclose(OD.solve_helmholtz_dirichlet(rhs, lam, dt, D), u, rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(OD.solve_poisson_dirichlet(A @ u, lam), u, rtol=1e-9, atol=1e-11)


def test_dct_oracle_pins():
    import scipy.fft
    from oracle import dst as OD
    rng = np.random.default_rng(1)
    for N in (1, 2, 5, 32, 100):
        x = rng.standard_normal((3, N))
        np.testing.assert_allclose(OD.dct2_ortho(x), scipy.fft.dct(x, type=2, norm="ortho", axis=-1),
                                   rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(OD.idct2_ortho(OD.dct2_ortho(x)), x, rtol=1e-12, atol=1e-12)
    # tests/test_fft_nonperiodic.py: Neumann symbol null mode, identity limit, constant kept
    lam = OD.laplacian_symbol_neumann(32, 0.1)
    assert abs(lam[0]) < 1e-14 and np.all(lam[1:] < 0)
    rhs = np.cos(np.pi * np.arange(32) / 32)
    # jnp.allclose defaults: rtol 1e-8 given, atol 1e-8
    np.testing.assert_allclose(OD.solve_helmholtz_neumann(rhs, lam, 1e-10, 1.0), rhs, rtol=1e-8, atol=1e-8)
    u = np.full(32, 5.0)
    for _ in range(10):
        u = OD.etd1_neumann(u, np.zeros(32), 0.1 * lam, 0.1)
    np.testing.assert_allclose(u, 5.0, rtol=1e-10, atol=1e-8)
    # the Helmholtz solve inverts (I - dt D Lap_N), the 3-point Laplacian with mirrored ends
    N, dx, dt, D = 40, 0.05, 0.2, 0.3
    A = (np.diag(-2.0 * np.ones(N)) + np.diag(np.ones(N - 1), 1) + np.diag(np.ones(N - 1), -1))
    A[0, 0] = A[-1, -1] = -1.0
    A /= dx ** 2
    v = rng.standard_normal(N)
    lamN = OD.laplacian_symbol_neumann(N, dx)
    np.testing.assert_allclose(OD.solve_helmholtz_neumann(v - dt * D * A @ v, lamN, dt, D), v,
                               rtol=1e-10, atol=1e-12)


# ------------------------------------------------------------- ETD1 / ETD2 / library ETDRK4
def _etd_case(n=128, L=1.0):
    from oracle import etd as OT
    dx = L / n
    x = (np.arange(n) + 0.5) * dx  # Grid1D interior coordinates (grid.py:87-110)
    return OT, x, dx


def test_etd1_zero_nonlinear_matches_exponential():
    # tests/test_fft_operators.py:393-422: ETD1 with N = 0 equals the pure exponential, < 1e-10
    OT, x, dx = _etd_case(128)
    lam = {"u": 0.1 * OT.fd_symbol_1d(128, dx)}
    state = {"u": np.sin(2 * np.pi * x)}
    for _ in range(int(0.1 / 0.01)):
        state = OT.etd1_step(state, 0.01, lam, OT.zero)
    pure = OT.diffusion_only_etd1(np.sin(2 * np.pi * x), 0.1, 0.01, lam["u"])
    assert np.linalg.norm(state["u"] - pure) / np.linalg.norm(pure) < 1e-10


def test_etd_integrate_api_pins():
    # tests/test_fft_operators.py:424-465: 5 saves, final state within 1e-3 of the exact decay
    OT, x, dx = _etd_case(128)
    D = 0.05
    t, hist = OT.etd_integrate({"u": np.sin(2 * np.pi * x)}, (0.0, 0.2), 0.01,
                               {"u": D * OT.fd_symbol_1d(128, dx)}, OT.zero, "etd1", 5)
    assert len(hist) == int(0.2 / 0.01 / 5) + 1
    exact = np.exp(-4 * np.pi ** 2 * D * 0.2) * np.sin(2 * np.pi * x)
    assert np.linalg.norm(hist[-1]["u"] - exact) / np.linalg.norm(exact) < 1e-3


def test_etdrk4_logistic_pins():
    # tests/test_fft_operators.py:517-559: ETDRK4 dt = 0.05 within 1 % of ETD1 dt = 0.001
    OT, x, dx = _etd_case(256)
    lam = {"u": 0.01 * OT.fd_symbol_1d(256, dx)}
    u0 = {"u": 0.5 + 0.3 * np.sin(2 * np.pi * x)}
    N_ = OT.logistic(0.1)
    _, h4 = OT.etd_integrate(u0, (0.0, 1.0), 0.05, lam, N_, "etdrk4")
    _, h1 = OT.etd_integrate(u0, (0.0, 1.0), 0.001, lam, N_, "etd1")
    rel = np.sqrt(np.mean((h4[-1]["u"] - h1[-1]["u"]) ** 2)) / np.sqrt(np.mean(h1[-1]["u"] ** 2))
    assert rel < 0.01


def test_etdrk4_library_order_pin():
    # tests/test_fft_operators.py:561-617: observed order > 3 (alpha = 0.5, t = 0.5)
    OT, x, dx = _etd_case(256)
    lam = {"u": 0.01 * OT.fd_symbol_1d(256, dx)}
    u0 = {"u": 0.5 + 0.3 * np.sin(2 * np.pi * x)}
    N_ = OT.logistic(0.5)
    ref = OT.etd_integrate(u0, (0.0, 0.5), 0.0001, lam, N_, "etdrk4")[1][-1]["u"]
    errs = [np.linalg.norm(OT.etd_integrate(u0, (0.0, 0.5), dt, lam, N_, "etdrk4")[1][-1]["u"] - ref)
            / np.linalg.norm(ref) for dt in (0.1, 0.05, 0.025, 0.0125)]
    orders = [np.log2(errs[i] / errs[i + 1]) for i in range(3) if errs[i + 1] > 1e-14]
    assert np.mean(orders) > 3.0


def test_etd2_second_order_and_phi_switch():
    OT, x, dx = _etd_case(128)
    lam = {"u": 0.01 * OT.fd_symbol_1d(128, dx)}
    u0 = {"u": 0.5 + 0.3 * np.sin(2 * np.pi * x)}
    N_ = OT.logistic(1.0)
    ref = OT.etd_integrate(u0, (0.0, 1.0), 0.001, lam, N_, "etdrk4")[1][-1]["u"]
    e = [np.linalg.norm(OT.etd_integrate(u0, (0.0, 1.0), dt, lam, N_, m)[1][-1]["u"] - ref)
         for m, dt in (("etd2", 0.1), ("etd2", 0.05), ("etd1", 0.1), ("etd1", 0.05))]
    assert 3.0 < e[0] / e[1] < 5.0   # ETD2: second order
    assert 1.6 < e[2] / e[3] < 2.5   # ETD1: first order
    # the Taylor branch and the closed form agree across |z| = 1e-4
    z = np.array([-0.99e-4, -1.01e-4])
    for f in (OT.phi1, OT.phi2):
        v = f(z)
        assert abs(v[0] - v[1]) < 1e-5 * abs(v[0])
    # L = 0: ETD1 is explicit Euler, ETD2 is Adams-Bashforth 2 (fft_integrators.py:172-174, 245-247)
    s0 = {"u": u0["u"]}
    e1 = OT.etd1_step(s0, 0.1, {"u": np.zeros(128)}, N_)
    assert np.allclose(e1["u"], u0["u"] + 0.1 * N_(s0)["u"], rtol=0, atol=1e-14)


@pytest.mark.parametrize("row", [r for r in _load("fft3d_published.json")["experiments"]
                                 if r["grid_size"] in (32, 48, 64, 80, 100)])
def test_fft3d_error_pins(row):
    # benchmarks/results/3d_feasibility.json: N^3, D = 0.1, 10 CN steps to T = 0.01, max error
    cfg = _load("fft3d_published.json")["config"]
    N_ = row["grid_size"]
    u0 = fftcn.node_grid_ic_3d(N_)
    dt = cfg["t_final"] / cfg["n_steps"]
    u = fftcn.fft_cn_3d(u0, cfg["D"], 1.0 / N_, dt, cfg["n_steps"])
    exact = u0 * np.exp(-12 * np.pi ** 2 * cfg["D"] * cfg["n_steps"] * dt)
    assert float(np.max(np.abs(u - exact))) == pytest.approx(row["error"], rel=1e-8)


def test_tubular_rk4_pins():
    # benchmarks/results/reactor_results.json: the penalty-BC RK4 sweep of
    # benchmark_tubular_reactor.py (N = 128, t_final = 15, 27 cases; the Robin cases equal the
    # Danckwerts ones).  The oracle's affine-power form is checked against its step loop, then
    # reproduces every published conversion, error and outlet value.
    from oracle import reactor as OR
    g = _load("tubular_published.json")
    dt, n = OR.tubular_dt(128, 10, 15.0)
    for bc in OR.TUBULAR_BCS:
        a = OR.tubular_rk4_loop(128, 10, 1.0, bc, dt, 300)
        b = OR.tubular_rk4(128, 10, 1.0, bc, dt, 300)
        assert np.max(np.abs(a - b)) < 1e-12
    for key, v in g["results"].items():
        dt, n = OR.tubular_dt(g["N"], v["Pe"], g["t_final"])
        assert n == v["n_steps"] and dt == pytest.approx(v["dt"], rel=1e-15)
        s = OR.tubular_summary(OR.tubular_rk4(g["N"], v["Pe"], v["Da"], v["bc_type"], dt, n),
                               v["Pe"], v["Da"], v["bc_type"], g["t_final"])
        for k in ("conversion", "error", "final_outlet_c"):
            assert s[k] == pytest.approx(v[k], rel=1e-8, abs=1e-40), (key, k)


def test_solver_comparison_1d_pins():
    # benchmarks/results/solver_comparison.json: 1D u_t = 0.01 u_xx - u_x, N = 1024, t in
    # [0, 10]; the max difference of FFT-CN (dt 1e-3) and of the exponential Strang IMEX
    # (dt 5e-3) from SciPy Radau (tests/golden/radau_advdiff1d.npy, made by
    # make_radau_advdiff1d.py; 568 output times, as published).
    g = _load("solver_comparison_published.json")
    ref = np.load(os.path.join(GOLD, "radau_advdiff1d.npy"))
    cfg = g["config"]
    n, D, v, T = cfg["N"], cfg["D"], cfg["v"], cfg["t_final"]
    u0 = fftcn.solver_comparison_ic(n)
    cn, imex_ = g["solvers"][1], g["solvers"][2]
    assert g["solvers"][0]["steps"] == 568
    u = fftcn.fft_cn_1d(u0, D, 1.0 / n, cn["dt"], cn["steps"], "spectral", v=v)
    assert float(np.max(np.abs(u - ref))) == pytest.approx(cn["error_vs_scipy"], rel=1e-6)
    u = fftcn.strang_exp_1d(u0, D, v, 1.0 / n, imex_["dt"], imex_["steps"])
    assert float(np.max(np.abs(u - ref))) == pytest.approx(imex_["error_vs_scipy"], rel=1e-6)
