"""Batched tubular-reactor CN and the 1D stencils vs the NumPy FP64 oracle."""

import json
import os

import numpy as np
import pytest
import torch

from oracle import mol
from oracle import reactor as OR

pytestmark = pytest.mark.gpu


def test_reactor_published_conversions(cuda):
    # benchmarks/results/method_comparison_results.json: CN, N=128, 100 steps of 0.05
    from moljax_gb300.core import reactor as R
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reactor_published.json")))
    for key, v in g["reactor_methods"].items():
        Pe = float(key.split()[0].split("=")[1])
        Da = float(key.split()[1].split("=")[1])
        c = R.tubular_reactor_cn(128, Pe, Da, v["CN"]["dt"], v["CN"]["steps"], "dirichlet", 0.0)
        assert 1 - float(c[-1]) == pytest.approx(v["CN"]["conversion"], rel=1e-10)


@pytest.mark.parametrize("variant", ["danckwerts", "dirichlet", "danckwerts_cn"])
def test_reactor_batch_uneven_vs_oracle(cuda, variant):
    from moljax_gb300.core import reactor as R
    rng = np.random.default_rng(5)
    kind = {"danckwerts": R.DANCKWERTS, "dirichlet": R.DIRICHLET, "danckwerts_cn": R.DANCKWERTS_CN}[variant]
    cases = []
    for n in (64, 100, 257, 1000, 4096):
        dt, ns = R.served_dt(n)
        if variant == "danckwerts":  # explicit upwind advection: stable for dt <= dz only
            dt = 0.5 / n
        ns = min(ns, 60)
        cases.append(R.ReactorCase(n, float(rng.uniform(10, 200)), float(rng.uniform(0.5, 5)), dt, ns, kind, 0.0))
    for dtype, tol in ((torch.float64, 1e-11), (torch.float32, 1e-4)):
        outs = R.solve_batch(cases, dtype)
        for c, o in zip(cases, outs):
            if variant == "danckwerts":
                ref = OR.danckwerts_cn(c.n, c.Pe, c.Da, c.dt, c.n_steps, c.c_init)
            elif variant == "danckwerts_cn":
                ref = OR.danckwerts_full_cn(c.n, c.Pe, c.Da, c.dt, c.n_steps, c.c_init)
            else:
                ref = OR.dirichlet_cn(c.n, c.Pe, c.Da, c.dt, c.n_steps, 1.0, c.c_init)
            # a stable run stays O(1) (CN overshoots the inlet value slightly, never grows)
            assert np.all(np.isfinite(ref)) and np.max(np.abs(ref)) <= 1.5
            err = np.linalg.norm(o.double().cpu().numpy() - ref) / np.linalg.norm(ref)
            assert err < tol, (c.n, err)


def test_reactor_alone_equals_in_batch(cuda):
    from moljax_gb300.core import reactor as R
    cases = [R.ReactorCase(n, 50.0, 2.0, *R.served_dt(n)) for n in (64, 512, 2048)]
    batch = R.solve_batch(cases, torch.float32)
    for c, b in zip(cases, batch):
        alone = R.solve_batch([c], torch.float32)[0]
        assert torch.equal(alone, b)


def test_stencil1d_vs_oracle(cuda):
    import moljax_gb300 as M
    g = M.Grid1D(40, 0.0, 2.0)
    og = mol.Grid1D(40, 0.0, 2.0)
    f = np.random.default_rng(0).standard_normal(42)
    ft = torch.tensor(f, device=cuda)
    np.testing.assert_allclose(M.laplacian_1d(ft, g).cpu().numpy(), mol.laplacian_1d(f, og), rtol=1e-13, atol=1e-11)
    for v in (1.5, -0.5):
        np.testing.assert_allclose(M.d1_upwind_1d(ft, v, g).cpu().numpy(), mol.d1_upwind_1d(f, v, og),
                                   rtol=1e-13, atol=1e-12)
    # README forms
    gr = M.Grid1D(n=128, L=1.0, bc_type="danckwerts")
    D2 = M.laplacian_1d(gr, order=2)
    D1 = M.gradient_1d(gr, upwind=True)
    c = torch.linspace(1, 0, 128, dtype=torch.float64, device=cuda)
    assert (D2 @ c).shape == (128,) and (D1 @ c).shape == (128,)
    assert float((D1 @ c)[0]) == pytest.approx((1.0 - 1.0) / gr.dx, abs=1e-9)


def test_tubular_rk4_sweep_published(cuda):
    """The 27-case penalty-RK4 sweep of benchmark_tubular_reactor.py (N = 128, t_final = 15, up
    to 967 740 RK4 steps per case) in one launch, FP64: every published conversion, error and
    outlet value (benchmarks/results/reactor_results.json) within 1e-8 relative, and the
    final profiles against the oracle within 1e-10."""
    from moljax_gb300.core import reactor as R
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "tubular_published.json")))
    res = R.run_tubular_sweep(N=g["N"], t_final=g["t_final"], dtype=torch.float64)
    assert set(res) == set(g["results"])
    for key, v in g["results"].items():
        r = res[key]
        assert r["n_steps"] == v["n_steps"]
        for k in ("conversion", "error", "final_outlet_c"):
            assert r[k] == pytest.approx(v[k], rel=1e-8, abs=1e-40), (key, k, r[k], v[k])
    # profiles against the oracle on uneven sizes (1 to 8 nodes per lane of a 4-warp CTA)
    cases, refs = [], []
    for n, bc, Pe, Da in ((3, "danckwerts", 5.0, 1.0), (37, "robin", 20.0, 2.0), (128, "neumann", 1.0, 0.5),
                          (257, "danckwerts", 50.0, 3.0), (512, "robin", 30.0, 1.5), (1000, "neumann", 200.0, 0.7),
                          (1024, "robin", 10.0, 4.0)):
        c = R.tubular_rk4_case(Pe, Da, bc, n, 0.5)
        c.n_steps = min(c.n_steps, 3000)
        cases.append(c)
        refs.append(OR.tubular_rk4_loop(n, Pe, Da, bc, c.dt, c.n_steps))
    for dtype, tol, nmax in ((torch.float64, 1e-12, 1024), (torch.float32, 2e-5, 1024)):
        sel = [i for i, c in enumerate(cases) if c.n <= nmax]
        outs = R.solve_batch([cases[i] for i in sel], dtype)
        for c, o, ref in zip([cases[i] for i in sel], outs, [refs[i] for i in sel]):
            err = float(np.max(np.abs(o.double().cpu().numpy() - ref)))
            assert err < tol * max(1.0, float(np.max(np.abs(ref)))), (c.n, c.variant, dtype, err)
