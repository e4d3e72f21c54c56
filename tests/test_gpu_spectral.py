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
