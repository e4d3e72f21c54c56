"""Periodic spectral operations on grids of any size (powers of two take the fused passes;
every other size the general full-spectrum path with Bluestein DFTs), against NumPy FFTs
of the reference's formulas (numpy / jnp.fft accept any n)."""

import numpy as np
import pytest
import torch

from oracle import fftcn
from oracle.mol import fd_symbol_1d, spectral_symbol_1d

pytestmark = pytest.mark.gpu

SHAPES = [(48, 80), (100, 100), (17, 33), (96, 128), (2000, 6), (5, 1)]


def _lam(ny, nx, dy, dx, kind):
    f = fd_symbol_1d if kind == "fd" else spectral_symbol_1d
    return f(ny, dy)[:, None] + f(nx, dx)[None, :]


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("kind", ["fd", "spectral"])
def test_general_multipliers_fp64(cuda, shape, kind):
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import get_plan
    ny, nx = shape
    dy, dx = 0.7 / ny, 1.3 / nx
    plan = get_plan(ny, nx, dy, dx, kind, torch.float64, cuda)
    assert getattr(plan, "general", False) == ((ny & (ny - 1)) != 0 or (nx & (nx - 1)) != 0 or nx < 2)
    rng = np.random.default_rng(ny * 7 + nx)
    u = rng.standard_normal((2, ny, nx))
    lam = _lam(ny, nx, dy, dx, kind)
    D, h = (0.05, 0.02), 0.01
    ut = torch.tensor(u, device=cuda)
    cases = {N.MULT_HELMHOLTZ: lambda d: 1 / (1 - h * d * lam), N.MULT_CN: lambda d: (1 + 0.5 * h * d * lam) / (1 - 0.5 * h * d * lam),
             N.MULT_EXP: lambda d: np.exp(h * d * lam), N.MULT_LAP: lambda d: h * d * lam}
    for mult, m in cases.items():
        got = plan.apply(ut, list(D), h, mult).cpu().numpy()
        for f in range(2):
            ref = np.real(np.fft.ifft2(m(D[f]) * np.fft.fft2(u[f])))
            assert float(np.max(np.abs(got[f] - ref))) < 1e-11 * max(1.0, float(np.max(np.abs(ref))))


def test_general_fp32_and_helpers(cuda):
    import moljax_gb300 as M
    ny, nx = 60, 90
    grid = M.Grid2D(nx, ny, 0.0, 1.0, 0.0, 0.8)
    rng = np.random.default_rng(1)
    u = rng.standard_normal((ny, nx))
    lam = _lam(ny, nx, grid.dy, grid.dx, "fd")
    # FP32 Helmholtz through the FFT cache of a non-power-of-two grid
    cache = M.create_fft_cache(grid, torch.float32)
    got = M.solve_helmholtz_2d(torch.tensor(u, dtype=torch.float32, device=cuda), cache.laplacian_symbol, 0.01, 0.1)
    ref = np.real(np.fft.ifft2(np.fft.fft2(u) / (1 - 0.001 * lam)))
    assert float(np.max(np.abs(got.cpu().double().numpy() - ref))) < 1e-5
    # FFT-CN (benchmark_vs_scipy.py:74-91 form) on 100 x 100, spectral symbol
    n = 100
    u0 = fftcn.node_grid_ic(n)
    cn = M.fft_cn_step(torch.tensor(u0, device=cuda), 0.1, 1.0 / n, 1e-3, 20).cpu().numpy()
    assert float(np.max(np.abs(cn - fftcn.fft_cn_2d(u0, 0.1, 1.0 / n, 1e-3, 20)))) < 1e-13
    # spectral filter with an arbitrary kernel
    K = rng.uniform(0, 1, (ny, nx))
    fl = M.apply_spectral_filter_interior(torch.tensor(u, device=cuda), torch.tensor(K)).cpu().numpy()
    np.testing.assert_allclose(fl, np.real(np.fft.ifft2(K * np.fft.fft2(u))), rtol=0, atol=1e-12)
    sig = M.exponential_filter_2d(ny, nx, 36.0, 8)
    fl2 = M.apply_spectral_filter_interior(torch.tensor(u, device=cuda), sig).cpu().numpy()
    np.testing.assert_allclose(fl2, np.real(np.fft.ifft2(sig.numpy() * np.fft.fft2(u))), rtol=0, atol=1e-12)


@pytest.mark.parametrize("n", [100, 90, 2047])
def test_general_1d_operators(cuda, n):
    import moljax_gb300 as M
    g = M.Grid1D.uniform(n, x_min=0.0, x_max=1.0)
    rng = np.random.default_rng(n)
    u = rng.standard_normal(n)
    ut = torch.tensor(u, device=cuda)
    uh = np.fft.fft(u)
    op = M.DiffusionOperator(g, 0.03)
    lam = 0.03 * fd_symbol_1d(n, g.dx)
    scale = max(1.0, float(np.max(np.abs(lam))))
    np.testing.assert_allclose(op.matvec(ut).cpu().numpy(), np.real(np.fft.ifft(lam * uh)), rtol=0, atol=1e-11 * scale)
    np.testing.assert_allclose(op.solve(ut, 0.2).cpu().numpy(), np.real(np.fft.ifft(uh / (1 - 0.2 * lam))), rtol=0, atol=1e-12)
    np.testing.assert_allclose(op.exp_matvec(ut, 0.2).cpu().numpy(), np.real(np.fft.ifft(np.exp(0.2 * lam) * uh)),
                               rtol=0, atol=1e-12)
    ad = M.AdvectionDiffusionOperator(g, v=1.3, D=0.01)
    lam_a = ad.eigenvalues.numpy()
    np.testing.assert_allclose(ad.solve(ut, 0.01).cpu().numpy(), np.real(np.fft.ifft(uh / (1 - 0.01 * lam_a))),
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(ad.exp_matvec(ut, 0.01).cpu().numpy(),
                               np.real(np.fft.ifft(np.exp(0.01 * lam_a) * uh)), rtol=0, atol=1e-12)
    np.testing.assert_allclose(ad.matvec(ut).cpu().numpy(), np.real(np.fft.ifft(lam_a * uh)), rtol=0,
                               atol=1e-11 * max(1.0, float(np.max(np.abs(lam_a)))))


@pytest.mark.parametrize("shape", [(48, 48), (30, 50)])
def test_imex_general_size_vs_oracle(cuda, shape):
    """adaptive_integrate_imex and the Strang / Euler / SSPRK2 steps on grids of other sizes
    against the FP64 oracle (identical accept/reject counts)."""
    import moljax_gb300 as M
    from oracle import imex as OI
    from oracle import mol
    ny, nx = shape
    grid = M.Grid2D(nx, ny, 0.0, 2.5, 0.0, 2.5)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, torch.float64, cuda)
    og = mol.Grid2D(nx, ny, 0, 2.5, 0, 2.5)
    y0 = mol.gray_scott_ic(og, 4)
    ym = {k: torch.tensor(v, device=cuda) for k, v in y0.items()}
    om, lam, od = OI.gray_scott_periodic(og, 2e-5, 1e-5, 0.035, 0.065)
    for fn, ofn in ((M.imex_strang_step, OI.imex_strang_step), (M.imex_euler_step, OI.imex_euler_step),
                    (M.imex_ssprk2_step, OI.imex_ssprk2_step)):
        a = fn(model, ym, 0.0, 0.8, cache, diff)
        b = ofn(om, y0, 0.8, lam, od)
        for k in ("u", "v"):
            assert float(np.max(np.abs(a[k].cpu().numpy() - b[k]))) < 1e-13
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 30.0, 1.0, cache, diff, pid_params=pid, save_every=1,
                                  max_steps=2000)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 30.0, 1.0, lam, od, pid=OI.PIDParams(atol=1e-7, rtol=1e-5),
                                    save_every=1, max_steps=2000)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    for k in ("u", "v"):
        assert float(np.max(np.abs(r.y_final[k].cpu().numpy() - ro.y_final[k]))) < 1e-10
    nh = ro.n_steps
    np.testing.assert_allclose(r.t_history.cpu().numpy()[:nh], ro.t_history[:nh], rtol=1e-9)
    with pytest.raises(NotImplementedError):
        M.adaptive_integrate_imex(model, ym, 0.0, 1.0, 0.1, cache, diff, precision="mixed")


@pytest.mark.parametrize("method", ["etd1", "etd2", "etdrk4"])
def test_etd_general_sizes_vs_oracle(cuda, method):
    import moljax_gb300 as M
    from oracle import etd as OT
    from oracle import etdrk4 as OE
    from oracle import mol
    # 1D logistic, n = 100
    g = M.Grid1D.uniform(100, x_min=0.0, x_max=1.0)
    x = g.x_coords().numpy()
    u0 = 0.5 + 0.3 * np.sin(2 * np.pi * x)
    _, h = M.etd_integrate({"u": torch.tensor(u0, device=cuda)}, (0.0, 0.5), 0.05, {"u": M.DiffusionOperator(g, 0.01)},
                           M.NativeNonlinear.logistic(0.5), method=method, save_every=5)
    _, ho = OT.etd_integrate({"u": u0}, (0.0, 0.5), 0.05, {"u": 0.01 * OT.fd_symbol_1d(100, g.dx)},
                             OT.logistic(0.5), method, 5)
    assert float(np.max(np.abs(h[-1]["u"].cpu().numpy() - ho[-1]["u"]))) < 1e-12
    # 2D coupled Gray-Scott on 40 x 48
    ny, nx, L = 40, 48, 2.5
    grid = M.Grid2D(nx, ny, 0.0, L, 0.0, L)
    og = mol.Grid2D(nx, ny, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 6)
    ui, vi = mol.interior(y0["u"], og), mol.interior(y0["v"], og)
    ops = {"u": M.DiffusionOperator(grid, 2e-5), "v": M.DiffusionOperator(grid, 1e-5)}
    _, h2 = M.etd_integrate({"u": torch.tensor(ui, device=cuda), "v": torch.tensor(vi, device=cuda)}, (0.0, 4.0), 1.0,
                            ops, M.NativeNonlinear.gray_scott(0.035, 0.065), method=method, save_every=4)
    lam = mol.fd_symbol_2d(ny, nx, og.dy, og.dx)
    _, h2o = OT.etd_integrate({"u": ui, "v": vi}, (0.0, 4.0), 1.0, {"u": 2e-5 * lam, "v": 1e-5 * lam},
                              OT.gray_scott(0.035, 0.065), method, 4, coupled=True)
    for f in ("u", "v"):
        assert float(np.max(np.abs(h2[-1][f].cpu().numpy() - h2o[-1][f]))) < 1e-12
    if method == "etdrk4":  # the benchmark's contour form on the MOLModel
        model = M.create_gray_scott_model(grid, 2e-5, 1e-5, 0.035, 0.065)
        out = M.etdrk4_gray_scott(model, {k: torch.tensor(v, device=cuda) for k, v in y0.items()}, 1.0, 4,
                                  variant="benchmark")
        ru, rv = OE.etdrk4_gray_scott(ui, vi, lam, 2e-5, 1e-5, 0.035, 0.065, 1.0, 4, 1.0)
        assert float(np.max(np.abs(mol.interior(out["u"].cpu().numpy(), og) - ru))) < 1e-12
        assert float(np.max(np.abs(mol.interior(out["v"].cpu().numpy(), og) - rv))) < 1e-12
