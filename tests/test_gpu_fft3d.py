"""Periodic 3D spectral passes on the GPU: the 3D FFT-CN of
benchmarks/sisc/bench_3d_feasibility.py against its published errors and the
NumPy oracle, and the general 3D multipliers on non-cubic boxes."""

import json
import os

import numpy as np
import pytest
import torch

from oracle import fftcn
from oracle.mol import fd_symbol_1d

pytestmark = pytest.mark.gpu
GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "fft3d_published.json")))


@pytest.mark.parametrize("n", [32, 48, 64, 80, 100, 128])
def test_fft_cn_3d_published_error(cuda, n):
    import moljax_gb300 as M
    cfg = GOLD["config"]
    row = next(r for r in GOLD["experiments"] if r["grid_size"] == n)
    u0 = fftcn.node_grid_ic_3d(n)
    dt = cfg["t_final"] / cfg["n_steps"]
    u = M.fft_cn_step_3d(torch.tensor(u0, device=cuda), cfg["D"], 1.0 / n, dt, cfg["n_steps"]).cpu().numpy()
    exact = u0 * np.exp(-12 * np.pi ** 2 * cfg["D"] * cfg["n_steps"] * dt)
    assert float(np.max(np.abs(u - exact))) == pytest.approx(row["error"], rel=1e-8)
    if n <= 80:
        ref = fftcn.fft_cn_3d(u0, cfg["D"], 1.0 / n, dt, cfg["n_steps"])
        assert float(np.max(np.abs(u - ref))) < 1e-14


def test_fft_cn_3d_fp32(cuda):
    import moljax_gb300 as M
    n = 64
    u0 = fftcn.node_grid_ic_3d(n)
    u = M.fft_cn_step_3d(torch.tensor(u0, dtype=torch.float32, device=cuda), 0.1, 1.0 / n, 1e-3, 10)
    ref = fftcn.fft_cn_3d(u0, 0.1, 1.0 / n, 1e-3, 10)
    assert float(np.max(np.abs(u.cpu().double().numpy() - ref))) < 2e-6


@pytest.mark.parametrize("shape", [(16, 32, 64), (64, 8, 32), (2, 4, 8)])
def test_multipliers_3d_noncubic(cuda, shape):
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import get_plan3d
    nz, ny, nx = shape
    dz, dy, dx = 0.7 / nz, 1.3 / ny, 0.9 / nx
    rng = np.random.default_rng(3)
    u = rng.standard_normal(shape)
    lam = (fd_symbol_1d(nz, dz)[:, None, None] + fd_symbol_1d(ny, dy)[None, :, None]
           + fd_symbol_1d(nx, dx)[None, None, :])
    uh = np.fft.fftn(u)
    plan = get_plan3d(nz, ny, nx, dz, dy, dx, "fd", torch.float64, cuda)
    ut = torch.tensor(u, device=cuda)
    D, h = 0.05, 0.01
    cases = {N.MULT_HELMHOLTZ: 1.0 / (1 - h * D * lam), N.MULT_EXP: np.exp(h * D * lam),
             N.MULT_CN: (1 + 0.5 * h * D * lam) / (1 - 0.5 * h * D * lam), N.MULT_LAP: h * D * lam}
    for mult, m in cases.items():
        ref = np.real(np.fft.ifftn(m * uh))
        got = plan.apply(ut, D, h, mult).cpu().numpy()
        assert float(np.max(np.abs(got - ref))) < 1e-12 * max(1.0, float(np.max(np.abs(ref))))
    # three applications = the cube of the multiplier
    got3 = plan.apply(ut, D, h, N.MULT_EXP, n_steps=3).cpu().numpy()
    np.testing.assert_allclose(got3, np.real(np.fft.ifftn(np.exp(3 * h * D * lam) * uh)), rtol=0, atol=1e-12)


def test_solve_helmholtz_3d(cuda):
    import moljax_gb300 as M
    n = 32
    rng = np.random.default_rng(5)
    f = rng.standard_normal((n, n, n))
    u = M.solve_helmholtz_3d(torch.tensor(f, device=cuda), 0.1, 0.01, 1.0 / n).cpu().numpy()
    lam = 3 * [fd_symbol_1d(n, 1.0 / n)]
    L = lam[0][:, None, None] + lam[1][None, :, None] + lam[2][None, None, :]
    np.testing.assert_allclose(u, np.real(np.fft.ifftn(np.fft.fftn(f) / (1 - 0.01 * 0.1 * L))), rtol=0, atol=1e-12)


@pytest.mark.parametrize("shape", [(12, 20, 36), (7, 16, 9)])
def test_general_box_multipliers(cuda, shape):
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import get_plan3d
    nz, ny, nx = shape
    dz, dy, dx = 0.7 / nz, 1.3 / ny, 0.9 / nx
    rng = np.random.default_rng(sum(shape))
    u = rng.standard_normal(shape)
    lam = (fd_symbol_1d(nz, dz)[:, None, None] + fd_symbol_1d(ny, dy)[None, :, None]
           + fd_symbol_1d(nx, dx)[None, None, :])
    plan = get_plan3d(nz, ny, nx, dz, dy, dx, "fd", torch.float64, cuda)
    assert plan.general
    ut = torch.tensor(u, device=cuda)
    uh = np.fft.fftn(u)
    for mult, m in {N.MULT_HELMHOLTZ: 1.0 / (1 - 0.01 * 0.05 * lam), N.MULT_EXP: np.exp(0.01 * 0.05 * lam)}.items():
        np.testing.assert_allclose(plan.apply(ut, 0.05, 0.01, mult).cpu().numpy(), np.real(np.fft.ifftn(m * uh)),
                                   rtol=0, atol=1e-12)
    np.testing.assert_allclose(plan.apply(ut, 0.05, 0.01, N.MULT_EXP, n_steps=3).cpu().numpy(),
                               np.real(np.fft.ifftn(np.exp(3 * 0.01 * 0.05 * lam) * uh)), rtol=0, atol=1e-12)
