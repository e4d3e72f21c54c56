"""FFT operators and spectral helpers on the GPU: the reference's own operator tests
(tests/test_fft_operators.py:66-383, 620-681) through the native path, and direct
parity of every multiplier against NumPy FFTs of the reference's formulas."""

import numpy as np
import pytest
import torch

from oracle import etd as OT

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _g1(n):
    import moljax_gb300 as M
    g = M.Grid1D.uniform(n, x_min=0.0, x_max=1.0)
    return g, g.x_coords().numpy()


def test_reference_diffusion_operator_cases(cuda):
    """test_diffusion_sinusoidal_decay, _multi_mode, _operator_matvec, _solve_consistency,
    test_spectral_bounds_exact, test_explicit_cfl_diffusion, test_etd_allows_large_dt,
    test_fft_vs_direct_helmholtz (tests/test_fft_operators.py:70-165, 211-236, 307-383)."""
    import moljax_gb300 as M
    g, x = _g1(128)
    op = M.DiffusionOperator(g, 0.01)
    u0 = torch.tensor(np.sin(2 * np.pi * x), device=cuda)
    uf = M.diffusion_only_etd1(u0, 1.0, 0.01, op).cpu().numpy()
    assert _rel(uf, np.exp(-4 * np.pi ** 2 * 0.01) * np.sin(2 * np.pi * x)) < 1e-4
    g2, x2 = _g1(256)
    u0m = np.sin(2 * np.pi * x2) + 0.5 * np.sin(4 * np.pi * x2) + 0.25 * np.sin(6 * np.pi * x2)
    um = M.diffusion_only_etd1(torch.tensor(u0m, device=cuda), 0.5, 0.005, M.DiffusionOperator(g2, 0.005))
    ex = (np.exp(-4 * np.pi ** 2 * 0.005 * 0.5) * np.sin(2 * np.pi * x2)
          + 0.5 * np.exp(-16 * np.pi ** 2 * 0.005 * 0.5) * np.sin(4 * np.pi * x2)
          + 0.25 * np.exp(-36 * np.pi ** 2 * 0.005 * 0.5) * np.sin(6 * np.pi * x2))
    assert _rel(um.cpu().numpy(), ex) < 1e-3
    op1 = M.DiffusionOperator(g, 1.0)
    Lu = op1.matvec(u0).cpu().numpy()
    assert _rel(Lu, -4 * np.pi ** 2 * np.sin(2 * np.pi * x)) < 0.01
    op = M.DiffusionOperator(g, 0.1)
    u = torch.tensor(np.sin(2 * np.pi * x) + 0.3 * np.cos(4 * np.pi * x), device=cuda)
    rec = op.solve(u - 0.01 * op.matvec(u), 0.01)
    assert _rel(rec.cpu().numpy(), u.cpu().numpy()) < 1e-10
    b = op.spectral_bounds()
    assert abs(b.rho - 4 * 0.1 / g.dx ** 2) / (4 * 0.1 / g.dx ** 2) < 0.01
    assert b.re_max <= 0.0 and b.im_max < 1e-10
    dt_cfl = M.exact_cfl_dt(op, method="explicit", safety=1.0)
    assert abs(dt_cfl - g.dx ** 2 / 0.2) / (g.dx ** 2 / 0.2) < 0.01
    ul = M.diffusion_only_etd1(u0, 0.1, 10 * dt_cfl, op).cpu().numpy()
    assert np.all(np.isfinite(ul))
    assert _rel(ul, np.exp(-4 * np.pi ** 2 * 0.1 * 0.1) * np.sin(2 * np.pi * x)) < 0.01
    rhs = torch.tensor(np.sin(2 * np.pi * x) + 0.5 * np.cos(6 * np.pi * x), device=cuda)
    cache = M.create_fft_cache(g)
    direct = M.solve_helmholtz_1d(rhs, cache.laplacian_symbol, 0.01, 0.1)
    assert _rel(op.solve(rhs, 0.01).cpu().numpy(), direct.cpu().numpy()) < 1e-12


def test_reference_advection_cases(cuda):
    """test_pure_advection_translation, test_advection_diffusion_eigenvalues
    (tests/test_fft_operators.py:169-210)."""
    import moljax_gb300 as M
    g, x = _g1(256)
    op = M.AdvectionDiffusionOperator(g, v=1.0, D=0.0)
    u = torch.tensor(np.sin(2 * np.pi * x), device=cuda)
    for _ in range(100):
        u = op.exp_matvec(u, 0.25 / 100)
    assert np.linalg.norm(u.cpu().numpy() - np.sin(2 * np.pi * (x - 0.25))) / np.linalg.norm(np.sin(2 * np.pi * x)) < 0.05
    g2, _ = _g1(128)
    lam = M.AdvectionDiffusionOperator(g2, v=2.0, D=0.1).eigenvalues
    assert float(lam.real.max()) <= 1e-10 and float(lam.imag.abs().max()) > 0


@pytest.mark.parametrize("n", [64, 256])
@pytest.mark.parametrize("D", [0.0, 0.02])
def test_advection_operator_1d_vs_numpy(cuda, n, D):
    import moljax_gb300 as M
    g, x = _g1(n)
    rng = np.random.default_rng(n)
    u = rng.standard_normal(n)
    op = M.AdvectionDiffusionOperator(g, v=1.3, D=D)
    lam = op.eigenvalues.numpy()
    uh = np.fft.fft(u)
    ut = torch.tensor(u, device=cuda)
    np.testing.assert_allclose(op.matvec(ut).cpu().numpy(), np.real(np.fft.ifft(lam * uh)), rtol=0, atol=1e-10)
    den = 1.0 - 0.01 * lam
    den = np.where(np.abs(den) < 1e-14, 1e-14, den)
    np.testing.assert_allclose(op.solve(ut, 0.01).cpu().numpy(), np.real(np.fft.ifft(uh / den)), rtol=0, atol=1e-12)
    np.testing.assert_allclose(op.exp_matvec(ut, 0.01).cpu().numpy(),
                               np.real(np.fft.ifft(np.exp(0.01 * lam) * uh)), rtol=0, atol=1e-12)


def test_advection_operator_2d_vs_numpy(cuda):
    import moljax_gb300 as M
    grid = M.Grid2D(32, 16, 0.0, 1.0, 0.0, 0.5)
    rng = np.random.default_rng(9)
    u = rng.standard_normal((16, 32))
    op = M.AdvectionDiffusionOperator(grid, v=(0.7, -1.1), D=0.01)
    lam = op.eigenvalues.cpu().numpy()
    uh = np.fft.fft2(u)
    ut = torch.tensor(u, device=cuda)
    np.testing.assert_allclose(op.matvec(ut).cpu().numpy(), np.real(np.fft.ifft2(lam * uh)), rtol=0, atol=1e-10)
    np.testing.assert_allclose(op.solve(ut, 0.02).cpu().numpy(), np.real(np.fft.ifft2(uh / (1 - 0.02 * lam))),
                               rtol=0, atol=1e-12)
    np.testing.assert_allclose(op.exp_matvec(ut, 0.02).cpu().numpy(),
                               np.real(np.fft.ifft2(np.exp(0.02 * lam) * uh)), rtol=0, atol=1e-12)


def test_spectral_filters_vs_numpy(cuda):
    import moljax_gb300 as M
    rng = np.random.default_rng(4)
    u = rng.standard_normal((32, 64))
    sig = M.exponential_filter_2d(32, 64, 36.0, 8)
    # fft_solvers.py:477-531 by hand
    def f1(n):
        k = np.arange(n)
        kn = np.minimum(np.minimum(k, n - k) / (n // 2), 1.0)
        return np.exp(-36.0 * kn ** 8)
    np.testing.assert_allclose(sig.numpy(), np.outer(f1(32), f1(64)), rtol=1e-15)
    out = M.apply_spectral_filter_interior(torch.tensor(u, device=cuda), sig).cpu().numpy()
    np.testing.assert_allclose(out, np.real(np.fft.ifft2(sig.numpy() * np.fft.fft2(u))), rtol=0, atol=1e-13)
    # an arbitrary (non-symmetric) real kernel: real(ifft2(K fft2(u)))
    K = rng.uniform(0.0, 1.0, (32, 64))
    out = M.apply_spectral_filter_interior(torch.tensor(u, device=cuda), torch.tensor(K)).cpu().numpy()
    np.testing.assert_allclose(out, np.real(np.fft.ifft2(K * np.fft.fft2(u))), rtol=0, atol=1e-13)
    # 1D and the padded / state forms
    g, x = _g1(128)
    u1 = rng.standard_normal(128)
    s1 = M.exponential_filter_1d(128, 10.0, 4)
    out1 = M.apply_spectral_filter_interior(torch.tensor(u1, device=cuda), s1).cpu().numpy()
    np.testing.assert_allclose(out1, np.real(np.fft.ifft(s1.numpy() * np.fft.fft(u1))), rtol=0, atol=1e-13)
    grid = M.Grid2D(64, 32, 0.0, 1.0, 0.0, 1.0)
    fp = torch.tensor(rng.standard_normal((34, 66)), device=cuda)
    st = M.apply_spectral_filter_state({"a": fp, "b": fp}, grid, sig, filter_fields={"b": False})
    np.testing.assert_allclose(st["a"][1:-1, 1:-1].cpu().numpy(),
                               np.real(np.fft.ifft2(sig.numpy() * np.fft.fft2(fp[1:-1, 1:-1].cpu().numpy()))),
                               rtol=0, atol=1e-13)
    assert torch.equal(st["a"][0], fp[0]) and torch.equal(st["b"], fp)


def test_diffusion_helpers_vs_numpy(cuda):
    import moljax_gb300 as M
    grid = M.Grid2D(64, 32, 0.0, 1.0, 0.0, 0.5)
    cache = M.create_fft_cache(grid)
    rng = np.random.default_rng(6)
    fp = torch.tensor(rng.standard_normal((34, 66)), device=cuda)
    lam = cache.laplacian_symbol.cpu().numpy()
    ui = fp[1:-1, 1:-1].cpu().numpy()
    sol = M.solve_diffusion_fft_field(fp, grid, 0.01, 0.3, cache)
    np.testing.assert_allclose(sol[1:-1, 1:-1].cpu().numpy(),
                               np.real(np.fft.ifft2(np.fft.fft2(ui) / (1 - 0.01 * 0.3 * lam))), rtol=0, atol=1e-13)
    assert torch.equal(sol[0], fp[0])
    st = M.apply_diffusion_fft({"u": fp, "w": fp}, grid, 0.01, {"u": 0.3}, cache)
    assert torch.equal(st["w"], fp) and torch.allclose(st["u"], sol, rtol=0, atol=1e-15)
    rhs = M.diffusion_rhs_fft({"u": fp, "w": fp}, grid, {"u": 0.3}, cache)
    np.testing.assert_allclose(rhs["u"][1:-1, 1:-1].cpu().numpy(), 0.3 * np.real(np.fft.ifft2(lam * np.fft.fft2(ui))),
                               rtol=0, atol=1e-9)
    assert float(rhs["u"][0].abs().max()) == 0.0 and float(rhs["w"].abs().max()) == 0.0
    # 1D
    g1, _ = _g1(64)
    c1 = M.create_fft_cache(g1)
    f1 = torch.tensor(rng.standard_normal(66), device=cuda)
    s1 = M.solve_diffusion_fft_field(f1, g1, 0.02, 0.1, c1)
    l1 = c1.laplacian_symbol.cpu().numpy()
    np.testing.assert_allclose(s1[1:-1].cpu().numpy(),
                               np.real(np.fft.ifft(np.fft.fft(f1[1:-1].cpu().numpy()) / (1 - 0.002 * l1))),
                               rtol=0, atol=1e-13)


def test_batched_and_stacked_solves(cuda):
    """test_batched_solve_matches_individual, test_stacked_solve_shared_op
    (tests/test_fft_operators.py:627-681), and the FFT IMEX-Euler step (545-585)."""
    import moljax_gb300 as M
    g, x = _g1(128)
    op = M.DiffusionOperator(g, 0.1)
    state = {"u": torch.tensor(np.sin(2 * np.pi * x), device=cuda),
             "v": torch.tensor(np.cos(4 * np.pi * x), device=cuda),
             "w": torch.tensor(np.sin(2 * np.pi * x) + 0.5 * np.cos(6 * np.pi * x), device=cuda)}
    ops = {"u": op, "v": op, "w": op}
    ind = {n: op.solve(r, 0.01) for n, r in state.items()}
    bat = M.batched_fft_solve(state, ops, 0.01)
    stk = M.stacked_fft_solve_shared_op(state, op, 0.01)
    for n in state:
        assert float((bat[n] - ind[n]).norm()) < 1e-12
        assert float((stk[n] - ind[n]).norm()) < 1e-12
    mv = M.batched_fft_matvec({"u": state["u"], "z": state["v"]}, {"u": op})
    assert float(mv["z"].abs().max()) == 0.0
    ex = M.batched_fft_exp_matvec(state, {"u": op}, 0.05)
    assert torch.equal(ex["v"], state["v"])
    from moljax_gb300.core.fft_integrators import imex_euler_step
    u0 = 0.5 + 0.3 * np.sin(2 * np.pi * x)
    out = imex_euler_step({"u": torch.tensor(u0, device=cuda)}, 0.0, 0.1, {"u": op},
                          M.NativeNonlinear.logistic(1.5))["u"].cpu().numpy()
    lam = 0.1 * OT.fd_symbol_1d(128, g.dx)
    rhs = u0 + 0.1 * 1.5 * u0 * (1 - u0)
    np.testing.assert_allclose(out, np.real(np.fft.ifft(np.fft.fft(rhs) / (1 - 0.1 * lam))), rtol=0, atol=1e-14)
