"""Parity at the benchmark configurations' own grid sizes.

The headline workloads run on grids the other parity tests only approach
with strips; here each runs at its full size against the NumPy FP64 oracle
over a bounded span (the oracle's cost is the limit, not the GPU's):

* Gray-Scott IMEX-Strang adaptive at 1024^2 (Du=2e-5, Dv=1e-5, F=0.035,
  k=0.065, L=2.5, rtol 1e-5, atol 1e-7, the seeded square-plus-noise initial
  condition, seed 20261203) over t in (0, 5): its first ~200 attempts, the
  stiff start-up transient where dt grows from 2e-3 to the CFL cap.  The
  mixed form (float-float spectral state) must take the oracle's accept/reject
  sequence and stay within rel-L2 1e-6; plain FP32 within 1e-4.
* Coupled Gray-Scott ETDRK4 at 2048^2 and 4096^2, FP32 state with FP64
  contour coefficients, dt = 1, three steps, rel-L2 <= 3e-6 per field.
* Newton-Krylov BDF2 of u_t = div((1+u^2) grad u) - u^3 at 512^2, Dirichlet,
  dt = 100 dx^2, three steps (BE first), rel-L2 <= 1e-7 and Newton counts
  within one of the oracle's.

The oracle's transforms use scipy.fft with every host core.
"""

import os

import numpy as np
import pytest
import torch

from oracle import etdrk4 as OE
from oracle import imex as OI
from oracle import mol
from oracle import nk as ONK

pytestmark = pytest.mark.gpu

GS = dict(Du=2e-5, Dv=1e-5, F=0.035, k=0.065)
SEED = 20261203


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def workers():
    w = os.cpu_count() or 1
    mol.set_fft_workers(w)
    OE.set_fft_workers(w)
    yield w
    mol.set_fft_workers(None)
    OE.set_fft_workers(None)


@pytest.fixture(scope="module")
def imex1024_oracle(workers):
    n, t_end = 1024, 5.0
    og = mol.Grid2D(n, n, 0, 2.5, 0, 2.5)
    y0 = mol.gray_scott_ic(og, SEED)
    om, lam, od = OI.gray_scott_periodic(og, GS["Du"], GS["Dv"], GS["F"], GS["k"])
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, t_end, 1.0, lam, od,
                                    pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=100000,
                                    max_steps=200000, keep_history=False)
    return og, y0, ro, t_end


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
def test_imex_strang_1024_vs_oracle(cuda, imex1024_oracle, precision):
    import moljax_gb300 as M
    og, y0, ro, t_end = imex1024_oracle
    assert ro.status == 0 and ro.n_accepted + ro.n_rejected >= 150
    grid = M.Grid2D(1024, 1024, 0.0, 2.5, 0.0, 2.5)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, GS["Du"], GS["Dv"], GS["F"], GS["k"],
                                                          torch.float32, cuda)
    ym = {k: torch.tensor(v, dtype=torch.float32, device=cuda) for k, v in y0.items()}
    r = M.adaptive_integrate_imex(model, ym, 0.0, t_end, 1.0, cache, diff,
                                  pid_params=M.PIDParams(atol=1e-7, rtol=1e-5), save_every=100000,
                                  max_steps=200000, save_y_history=False, precision=precision)
    assert r.status == 0
    errs = [_rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) for k in ("u", "v")]
    if precision == "mixed":
        assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
        assert max(errs) < 1e-6, errs
    else:
        assert abs(r.n_accepted - ro.n_accepted) <= 2 and abs(r.n_rejected - ro.n_rejected) <= 2
        assert max(errs) < 1e-4, errs


@pytest.mark.parametrize("n", [2048, 4096])
def test_etdrk4_full_size_vs_oracle(cuda, workers, n):
    import moljax_gb300 as M
    L, dt, steps = 2.5, 1.0, 3
    grid = M.Grid2D(n, n, 0.0, L, 0.0, L)
    model = M.create_gray_scott_model(grid, GS["Du"], GS["Dv"], GS["F"], GS["k"], dtype=torch.float32)
    og = mol.Grid2D(n, n, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, SEED)
    ym = {k: torch.tensor(v, dtype=torch.float32, device=cuda) for k, v in y0.items()}
    out = M.etdrk4_gray_scott(model, ym, dt, steps)
    gu = mol.interior(out["u"].cpu().numpy(), og)
    gv = mol.interior(out["v"].cpu().numpy(), og)
    del out, ym
    ly, lx = mol.fd_symbol_1d(n, og.dy), mol.fd_symbol_1d(n, og.dx)
    cu = OE.etdrk4_coeffs_separable(ly, lx, GS["Du"], dt, workers=workers)
    cv = OE.etdrk4_coeffs_separable(ly, lx, GS["Dv"], dt, workers=workers)
    u, v = mol.interior(y0["u"], og).copy(), mol.interior(y0["v"], og).copy()
    for _ in range(steps):
        u, v = OE.etdrk4_step(u, v, cu, cv, GS["F"], GS["k"], 2.0)
    eu, ev = _rel(gu, u), _rel(gv, v)
    assert eu < 3e-6 and ev < 3e-6, (eu, ev)


def test_nk_bdf2_512_vs_oracle(cuda):
    import moljax_gb300 as M
    n = 512
    dx = 1.0 / n
    dt = 100 * dx * dx
    u0 = ONK.gaussians_ic(n)
    u, st = M.integrate_implicit_vardiff(torch.tensor(u0, device=cuda), dx, dt, 3, method="bdf2",
                                         nk_params=M.NKParams(gmres_restart=30), be_guess="previous")
    ref, rst = ONK.bdf2_integrate(u0, dx, dx, dt, 3, restart=30, be_guess="previous")
    assert bool(st[:, 2].all()) and all(bool(s[2]) for s in rst)
    assert _rel(u.cpu().numpy(), ref) < 1e-7
    assert np.max(np.abs(st[:, 0].numpy() - np.array([s[0] for s in rst]))) <= 1
