"""Spectral passes on the GPU vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import fftcn, mol

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("ny,nx", [(2, 2), (4, 8), (16, 16), (32, 64), (128, 128), (256, 32),
                                   (64, 1024), (512, 512), (4096, 16), (16, 4096)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_helmholtz_vs_oracle(cuda, ny, nx, dtype):
    from moljax_gb300.core import fft_solvers
    rng = np.random.default_rng(ny * 7 + nx)
    dy, dx = 2.5 / ny, 2.5 / nx
    rhs = rng.standard_normal((3, ny, nx))
    D = [2e-5, 1e-5, 0.3]
    plan = fft_solvers.get_plan(ny, nx, dy, dx, "fd", dtype, cuda)
    out = plan.apply(torch.tensor(rhs, dtype=dtype, device=cuda), D, 0.7, 1).cpu().numpy()
    lam = mol.fd_symbol_2d(ny, nx, dy, dx)
    tol = 1e-13 if dtype == torch.float64 else 3e-6
    for f in range(3):
        ref = mol.solve_helmholtz_2d(rhs[f], lam, 0.7, D[f])
        assert _rel(out[f], ref) < tol


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_roundtrip_identity(cuda, dtype):
    from moljax_gb300.core import fft_solvers
    rng = np.random.default_rng(5)
    x = rng.standard_normal((2, 256, 128))
    plan = fft_solvers.get_plan(256, 128, 0.1, 0.1, "fd", dtype, cuda)
    out = plan.apply(torch.tensor(x, dtype=dtype, device=cuda), [1.0, 1.0], 0.0, 0).cpu().numpy()
    tol = 1e-14 if dtype == torch.float64 else 1e-6
    assert _rel(out, x) < tol


def test_zero_diffusivity_passes_through(cuda):
    # fft_solvers.py:435-443 / tests/test_fft_solver.py:253-279
    from moljax_gb300.core import fft_solvers
    x = torch.randn(2, 32, 32, dtype=torch.float64, device=cuda)
    plan = fft_solvers.get_plan(32, 32, 0.1, 0.1, "fd", torch.float64, cuda)
    out = plan.apply(x, [0.0, 0.5], 0.1, 1)
    assert torch.equal(out[0], x[0])
    assert not torch.equal(out[1], x[1])


def test_fft_cn_config1_fp64(cuda):
    # 128^2 on [0,1)^2, D=0.1, dt=0.01, 100 steps one by one; spectral symbol
    from moljax_gb300.core import fft_solvers
    u0 = fftcn.node_grid_ic(128)
    u = fft_solvers.fft_cn_step(torch.tensor(u0, device=cuda), 0.1, 1 / 128, 0.01, n_steps=100)
    u = u.cpu().numpy()
    ref = fftcn.fft_cn_2d(u0, 0.1, 1 / 128, 0.01, 100)
    assert _rel(u, ref) < 1e-12
    ana = fftcn.analytic_decay(u0, 0.1, 1.0)
    assert _rel(u, ana) < 5e-3  # CN truncation (4.10e-3)


def test_fft_cn_published_table(cuda):
    # benchmarks/results/precision_fp32_fp64.json, FP64 rows, through the GPU path
    import json, os
    from moljax_gb300.core import fft_solvers
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "fftcn_published.json")))
    u0 = fftcn.node_grid_ic(128)
    D, T = g["precision_table"]["D"], g["precision_table"]["t_final"]
    for row in g["precision_table"]["fp64"][:4]:
        n = row["n_steps"]
        u = fft_solvers.fft_cn_step(torch.tensor(u0, device=cuda), D, 1 / 128, row["dt"], n)
        err = np.max(np.abs(u.cpu().numpy() - fftcn.analytic_decay(u0, D, n * row["dt"])))
        assert err == pytest.approx(row["error"], rel=1e-6)


def test_fft_cn_fd_symbol(cuda):
    from moljax_gb300.core import fft_solvers
    u0 = fftcn.node_grid_ic(64)
    u = fft_solvers.fft_cn_step(torch.tensor(u0, device=cuda), 0.1, 1 / 64, 0.01, 10, symbol="fd")
    ref = fftcn.fft_cn_2d(u0, 0.1, 1 / 64, 0.01, 10, kind="fd")
    assert _rel(u.cpu().numpy(), ref) < 1e-12


def test_solver_comparison_1d_published(cuda):
    """benchmarks/results/solver_comparison.json through the native 1D advection-diffusion
    path (N = 1024, D = 0.01, v = 1, t = 10, FP64): FFT-CN (dt 1e-3, 10 000 steps) and the
    exponential Strang IMEX (dt 5e-3, 2 000 steps) reproduce the published max differences
    from SciPy Radau (tests/golden/radau_advdiff1d.npy) and the oracle's final states."""
    import json
    import os
    import moljax_gb300 as M
    gold = os.path.join(os.path.dirname(__file__), "golden")
    g = json.load(open(os.path.join(gold, "solver_comparison_published.json")))
    ref = np.load(os.path.join(gold, "radau_advdiff1d.npy"))
    cfg = g["config"]
    n, D, v, T = cfg["N"], cfg["D"], cfg["v"], cfg["t_final"]
    u0 = fftcn.solver_comparison_ic(n)
    cn, im = g["solvers"][1], g["solvers"][2]
    ut = torch.tensor(u0, device=cuda)
    u = M.fft_cn_advdiff_1d(ut, D, v, 1.0 / n, cn["dt"], cn["steps"]).cpu().numpy()
    assert float(np.max(np.abs(u - ref))) == pytest.approx(cn["error_vs_scipy"], rel=1e-5)
    o = fftcn.fft_cn_1d(u0, D, 1.0 / n, cn["dt"], cn["steps"], "spectral", v=v)
    assert float(np.max(np.abs(u - o))) < 1e-12
    u = M.imex_advdiff_1d(ut, D, v, 1.0 / n, im["dt"], im["steps"]).cpu().numpy()
    assert float(np.max(np.abs(u - ref))) == pytest.approx(im["error_vs_scipy"], rel=1e-5)
    o = fftcn.strang_exp_1d(u0, D, v, 1.0 / n, im["dt"], im["steps"])
    assert float(np.max(np.abs(u - o))) < 1e-12
    # a length that is not a power of two takes the general path with the same results
    m = 768
    w0 = fftcn.solver_comparison_ic(m)
    w = M.fft_cn_advdiff_1d(torch.tensor(w0, device=cuda), D, v, 1.0 / m, 1e-3, 200).cpu().numpy()
    assert float(np.max(np.abs(w - fftcn.fft_cn_1d(w0, D, 1.0 / m, 1e-3, 200, "spectral", v=v)))) < 1e-12
    w = M.imex_advdiff_1d(torch.tensor(w0, device=cuda), D, v, 1.0 / m, 5e-3, 100).cpu().numpy()
    assert float(np.max(np.abs(w - fftcn.strang_exp_1d(w0, D, v, 1.0 / m, 5e-3, 100)))) < 1e-12
