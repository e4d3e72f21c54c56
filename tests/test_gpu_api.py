"""The rest of the reference's path API on the GPU: variable-coefficient diffusion
(tests/test_variable_coeff.py:98-165 and the formula), second-derivative stencils,
operator factories, step-doubling helpers and the implicit residual factories, each
against the NumPy oracle or the reference's formulas."""

import numpy as np
import pytest
import torch

from oracle import imex as OI
from oracle import mol
from oracle import explicit as OX

pytestmark = pytest.mark.gpu


def _vardiff_np(u, D, dy, dx, ng, ny, nx):
    """variable_coeff.py:232-287 restated."""
    if D.shape == (ny, nx):
        D = np.pad(D, ng, mode="edge")
    out = np.zeros_like(u)
    c = (slice(ng, ng + ny), slice(ng, ng + nx))
    Dc = D[c]
    dxp = 0.5 * (Dc + D[ng:ng + ny, ng + 1:ng + nx + 1])
    dxm = 0.5 * (Dc + D[ng:ng + ny, ng - 1:ng + nx - 1])
    dyp = 0.5 * (Dc + D[ng + 1:ng + ny + 1, ng:ng + nx])
    dym = 0.5 * (Dc + D[ng - 1:ng + ny - 1, ng:ng + nx])
    uc = u[c]
    Lx = (dxp * (u[ng:ng + ny, ng + 1:ng + nx + 1] - uc) - dxm * (uc - u[ng:ng + ny, ng - 1:ng + nx - 1])) / dx ** 2
    Ly = (dyp * (u[ng + 1:ng + ny + 1, ng:ng + nx] - uc) - dym * (uc - u[ng - 1:ng + ny - 1, ng:ng + nx])) / dy ** 2
    out[c] = Lx + Ly
    return out


@pytest.mark.parametrize("dshape", ["padded", "interior"])
def test_variable_diffusion_2d(cuda, dshape):
    import moljax_gb300 as M
    ny, nx, ng = 48, 64, 1
    rng = np.random.default_rng(2)
    u = rng.standard_normal((ny + 2, nx + 2))
    D = 1.0 + rng.uniform(0, 1, (ny + 2, nx + 2) if dshape == "padded" else (ny, nx))
    got = M.apply_variable_diffusion_2d(torch.tensor(u, device=cuda), torch.tensor(D, device=cuda),
                                        0.03, 0.02, ng, ny, nx).cpu().numpy()
    np.testing.assert_allclose(got, _vardiff_np(u, D, 0.03, 0.02, ng, ny, nx), rtol=1e-12, atol=1e-9)


def test_reference_variable_diffusion_cases(cuda):
    """tests/test_variable_coeff.py:100-165: constant D = the Laplacian (1D, 2D)."""
    import moljax_gb300 as M
    n, ng = 64, 1
    dx = 2 * np.pi / n
    x = np.linspace(-ng * dx, 2 * np.pi + ng * dx, n + 2 * ng, endpoint=False)
    u = np.sin(x)
    Lu = M.variable_coeff.apply_variable_diffusion_1d(torch.tensor(u, device=cuda),
                                                      torch.full((n + 2,), 2.0, device=cuda, dtype=torch.float64),
                                                      dx, ng, n).cpu().numpy()
    assert np.max(np.abs(Lu[ng:ng + n] - (-2.0 * np.sin(x))[ng:ng + n])) < 0.01
    L = 2 * np.pi
    xx = np.linspace(0, L, 66, endpoint=False)
    X, Y = np.meshgrid(xx, xx)
    u2 = np.sin(X) * np.sin(Y)
    Lu2 = M.apply_variable_diffusion_2d(torch.tensor(u2, device=cuda), torch.ones(66, 66, device=cuda, dtype=torch.float64),
                                        L / 64, L / 64, 1, 64, 64).cpu().numpy()
    assert np.max(np.abs(Lu2[1:-1, 1:-1] - (-2.0 * u2)[1:-1, 1:-1])) < 0.5


def test_second_derivative_stencils_and_factories(cuda):
    import moljax_gb300 as M
    grid = M.Grid2D(32, 24, 0.0, 1.0, 0.0, 0.75)
    og = mol.Grid2D(32, 24, 0, 1.0, 0, 0.75)
    rng = np.random.default_rng(8)
    f = rng.standard_normal((26, 34))
    ft = torch.tensor(f, device=cuda)
    for axis, d in ((0, grid.dy), (1, grid.dx)):
        got = M.d2_central_2d(ft, grid, axis).cpu().numpy()
        ref = np.zeros_like(f)
        if axis == 0:
            ref[1:-1, 1:-1] = (f[2:, 1:-1] - 2 * f[1:-1, 1:-1] + f[:-2, 1:-1]) / d ** 2
        else:
            ref[1:-1, 1:-1] = (f[1:-1, 2:] - 2 * f[1:-1, 1:-1] + f[1:-1, :-2]) / d ** 2
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-8)
    st = {"c": ft, "d": ft * 2}
    params = {"D": 0.3, "vx": 0.7, "vy": -0.4}
    dif = M.make_diffusion_op_2d("c").apply(st, grid, 0.0, params)
    adv = M.make_advection_op_2d("c").apply(st, grid, 0.0, params)
    tot = M.op_sum([M.make_diffusion_op_2d("c"), M.make_advection_op_2d("c")])(st, grid, 0.0, params)
    lap = 0.3 * mol.laplacian_2d(f, og)
    up = -0.7 * mol.d1_upwind_2d(f, 0.7, og, 1) + 0.4 * mol.d1_upwind_2d(f, -0.4, og, 0)
    np.testing.assert_allclose(dif["c"].cpu().numpy(), lap, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(adv["c"].cpu().numpy(), up, rtol=1e-12, atol=1e-9)
    np.testing.assert_allclose(tot["c"].cpu().numpy(), lap + up, rtol=1e-12, atol=1e-9)
    assert float(dif["d"].abs().max()) == 0.0
    rx = M.make_reaction_op({"c": lambda s, p: s["c"] * p["D"]}).apply(st, grid, 0.0, params)
    assert torch.allclose(rx["c"], 0.3 * ft) and float(rx["d"].abs().max()) == 0.0


def test_step_doubling_helpers_vs_oracle(cuda):
    import moljax_gb300 as M
    n = 32
    grid = M.Grid2D(n, n, 0.0, 2.5, 0.0, 2.5)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, torch.float64, cuda)
    og = mol.Grid2D(n, n, 0, 2.5, 0, 2.5)
    y0 = mol.gray_scott_ic(og, 3)
    ym = {k: torch.tensor(v, device=cuda) for k, v in y0.items()}
    om, lam, od = OI.gray_scott_periodic(og, 2e-5, 1e-5, 0.035, 0.065)
    yh, err = M.estimate_error_imex_doubling(model, ym, 0.0, 0.8, cache, diff)
    ryh, rerr = OI.estimate_error_imex_doubling(om, y0, 0.8, lam, od)
    for k in ("u", "v"):
        np.testing.assert_allclose(yh[k].cpu().numpy(), ryh[k], rtol=0, atol=1e-13)
        np.testing.assert_allclose(err[k].cpu().numpy(), rerr[k], rtol=0, atol=1e-13)
    # explicit step doubling on the advection-diffusion model
    gm = M.create_advection_diffusion_model(grid, field_names=("c",), D=1e-3, vx=0.3, vy=-0.2,
                                            dtype=torch.float64)
    st = {"c": torch.tensor(y0["u"], device=cuda)}
    xm = OX.ExplicitModel(og, {"c": 0}, {"c": 1e-3}, vx=0.3, vy=-0.2, advection="upwind",
                          params={"D": 1e-3, "vx": 0.3, "vy": -0.2})
    # interiors: the native steps return the ghosts filled by the BCs, the oracle's axpy
    # keeps the input ghosts; every use of a state re-applies the BCs first
    c = (slice(1, -1), slice(1, -1))
    for method in (0, 1, 2):
        yh, err = M.step_explicit_with_error(gm, st, 0.0, 0.01, method)
        ry, re = OX.step_explicit_with_error(xm, {"c": y0["u"]}, 0.01, method)
        np.testing.assert_allclose(yh["c"].cpu().numpy()[c], ry["c"][c], rtol=0, atol=1e-12)
        np.testing.assert_allclose(err["c"].cpu().numpy()[c], re["c"][c], rtol=0, atol=1e-12)
        one = M.step_explicit(gm, st, 0.0, 0.01, method)["c"].cpu().numpy()
        np.testing.assert_allclose(one[c], OX.STEPS[method](xm, {"c": y0["u"]}, 0.01)["c"][c], rtol=0, atol=1e-12)


def test_implicit_residual_factories(cuda):
    import moljax_gb300 as M
    n = 16
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_gray_scott_model(grid, 2e-3, 1e-3, 0.035, 0.065)
    og = mol.Grid2D(n, n, 0, 1.0, 0, 1.0)
    ya, yb, yc = (mol.gray_scott_ic(og, s) for s in (1, 2, 3))
    T = {k: torch.tensor(v, device=cuda) for k, v in ya.items()}
    Tb = {k: torch.tensor(v, device=cuda) for k, v in yb.items()}
    Tc = {k: torch.tensor(v, device=cuda) for k, v in yc.items()}
    F = lambda y: {k: v.cpu().numpy() for k, v in model.rhs(y, 0.0).items()}  # noqa: E731
    Fa, Fb = F(T), F(Tb)
    r = M.create_implicit_residual(model, Tb, 0.1, 0.1, "be")(T)
    r2 = M.create_implicit_residual(model, Tb, 0.1, 0.1, "cn")(T)
    w = 0.1 / 0.07
    a0, a1, a2, beta = (1 + 2 * w) / (1 + w), -(1 + w), w * w / (1 + w), 0.1 * (1 + w) / (1 + 2 * w)
    r3 = M.create_bdf2_residual(model, Tb, Tc, 0.2, 0.1, 0.07)(T)
    for k in ("u", "v"):
        np.testing.assert_allclose(r[k].cpu().numpy(), ya[k] - yb[k] - 0.1 * Fa[k], rtol=0, atol=1e-14)
        np.testing.assert_allclose(r2[k].cpu().numpy(), ya[k] - yb[k] - 0.05 * (Fb[k] + Fa[k]), rtol=0, atol=1e-14)
        np.testing.assert_allclose(r3[k].cpu().numpy(), a0 * ya[k] + a1 * yb[k] + a2 * yc[k] - beta * Fa[k],
                                   rtol=0, atol=1e-13)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_imex_ssprk2_step_vs_oracle(cuda, dtype):
    import moljax_gb300 as M
    n = 64
    grid = M.Grid2D(n, n, 0.0, 2.5, 0.0, 2.5)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, dtype, cuda)
    og = mol.Grid2D(n, n, 0, 2.5, 0, 2.5)
    y0 = mol.gray_scott_ic(og, 13)
    om, lam, od = OI.gray_scott_periodic(og, 2e-5, 1e-5, 0.035, 0.065)
    y = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
    yo = y0
    for _ in range(3):
        y = M.imex_ssprk2_step(model, y, 0.0, 0.7, cache, diff)
        yo = OI.imex_ssprk2_step(om, yo, 0.7, lam, od)
    tol = 1e-13 if dtype == torch.float64 else 2e-6
    for k in ("u", "v"):
        r = float(np.linalg.norm(y[k].cpu().double().numpy() - yo[k]) / np.linalg.norm(yo[k]))
        assert r < tol  # ghosts included (periodic fill)
