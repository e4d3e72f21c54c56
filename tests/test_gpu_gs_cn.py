"""Crank-Nicolson Gray-Scott by the preconditioned Newton iteration of the reference's
Gray-Scott benchmark (device-side Newton loop) vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import gs_cn as G

pytestmark = pytest.mark.gpu

P = dict(Du=2e-5, Dv=1e-5, F=0.035, k=0.065)


@pytest.mark.parametrize("n,steps", [(64, 10), (256, 4)])
def test_gs_cn_newton_vs_oracle(cuda, n, steps):
    import moljax_gb300 as M
    u0, v0 = G.benchmark_ic(n)  # benchmarks/benchmark_gray_scott.py:60-62
    dx = 1.0 / n
    u, v, its = M.gray_scott_cn_newton(torch.tensor(u0, device=cuda), torch.tensor(v0, device=cuda), dt=0.5,
                                       n_steps=steps, dx=dx, **P)
    ru, rv, rits = G.cn_solve(u0, v0, G.spectral_symbol(n, dx), P["Du"], P["Dv"], P["F"], P["k"], 0.5, steps)
    assert its.cpu().tolist() == rits
    for a, b in ((u, ru), (v, rv)):
        assert float(np.linalg.norm(a.cpu().numpy() - b) / np.linalg.norm(b)) < 1e-11


def test_gs_cn_newton_iteration_cap_and_fd_symbol(cuda):
    """max_iter caps every step; the FD symbol option follows the same oracle."""
    import moljax_gb300 as M
    from oracle import mol
    n = 32
    u0, v0 = G.benchmark_ic(n)
    dx = 1.0 / n
    u, v, its = M.gray_scott_cn_newton(torch.tensor(u0, device=cuda), torch.tensor(v0, device=cuda), dt=0.5,
                                       n_steps=3, dx=dx, max_iter=2, symbol="fd", **P)
    lam = mol.fd_symbol_2d(n, n, dx, dx)
    ru, rv, rits = G.cn_solve(u0, v0, lam, P["Du"], P["Dv"], P["F"], P["k"], 0.5, 3, max_iter=2)
    assert its.cpu().tolist() == rits == [2, 2, 2]
    assert float(np.linalg.norm(u.cpu().numpy() - ru) / np.linalg.norm(ru)) < 1e-11


@pytest.mark.parametrize("n,steps", [(64, 40), (256, 12)])
def test_gs_strang_exp_vs_oracle(cuda, n, steps):
    """The benchmark's Strang exp-diffusion IMEX (imex_step, benchmark_gray_scott.py:268-296)
    against the oracle, FP64, pseudo-spectral; steps beyond one graph of 64 and below it."""
    import moljax_gb300 as M
    u0, v0 = G.benchmark_ic(n)
    dx = 1.0 / n
    lam = G.spectral_symbol(n, dx)
    for st in (1, steps, 130):
        u, v = M.gray_scott_strang_exp(torch.tensor(u0, device=cuda), torch.tensor(v0, device=cuda),
                                       P["Du"], P["Dv"], P["F"], P["k"], 0.5, st, dx)
        ru, rv = G.strang_exp_solve(u0, v0, lam, P["Du"], P["Dv"], P["F"], P["k"], 0.5, st)
        for a, b in ((u, ru), (v, rv)):
            assert float(np.linalg.norm(a.cpu().numpy() - b) / np.linalg.norm(b)) < 1e-12, st
    # the benchmark's initial condition as the package builds it equals the oracle's
    from moljax_gb300.workloads import gray_scott_benchmark_ic
    uu, vv = gray_scott_benchmark_ic(n, torch.float64, cuda)
    assert np.array_equal(uu.cpu().numpy(), u0) and np.array_equal(vv.cpu().numpy(), v0)


@pytest.mark.parametrize("n,steps", [(64, 40), (256, 20)])
def test_gs_rk4_spectral_vs_oracle(cuda, n, steps):
    """The benchmark's pseudo-spectral RK4 (rk4_step, benchmark_gray_scott.py:93-131) at
    0.9 of its stability limit against the oracle, FP64; a run longer than one 16-step graph
    and one shorter."""
    import moljax_gb300 as M
    u0, v0 = G.benchmark_ic(n)
    dx = 1.0 / n
    lam = G.spectral_symbol(n, dx)
    dt = G.rk4_dt(n, P["Du"], P["Dv"], dx)
    for st in (3, steps):
        u, v = M.gray_scott_rk4_spectral(torch.tensor(u0, device=cuda), torch.tensor(v0, device=cuda),
                                         P["Du"], P["Dv"], P["F"], P["k"], dt, st, dx)
        ru, rv = G.rk4_solve(u0, v0, lam, P["Du"], P["Dv"], P["F"], P["k"], dt, st)
        for a, b in ((u, ru), (v, rv)):
            assert float(np.linalg.norm(a.cpu().numpy() - b) / np.linalg.norm(b)) < 1e-12, st
