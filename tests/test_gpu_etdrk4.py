"""Coupled Gray-Scott ETDRK4 on the GPU vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import etdrk4 as OE
from oracle import mol

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n,symbol,variant", [(32, "fd", "cox-matthews"), (64, "spectral", "benchmark"),
                                              (128, "fd", "benchmark"), (64, "fd", "cox-matthews")])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_etdrk4_vs_oracle(cuda, n, symbol, variant, dtype):
    import moljax_gb300 as M
    L = 2.5
    grid = M.Grid2D(n, n, 0.0, L, 0.0, L)
    model = M.create_gray_scott_model(grid, 2e-5, 1e-5, 0.035, 0.065, dtype=dtype)
    og = mol.Grid2D(n, n, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 7)
    ym = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
    out = M.etdrk4_gray_scott(model, ym, 1.0, 10, symbol=symbol, variant=variant)
    lam = (mol.fd_symbol_2d if symbol == "fd" else mol.spectral_symbol_2d)(n, n, og.dy, og.dx)
    ru, rv = OE.etdrk4_gray_scott(mol.interior(y0["u"], og), mol.interior(y0["v"], og), lam,
                                  2e-5, 1e-5, 0.035, 0.065, 1.0, 10,
                                  2.0 if variant == "cox-matthews" else 1.0)
    tol = 1e-11 if dtype == torch.float64 else 3e-6
    assert _rel(mol.interior(out["u"].cpu().numpy(), og), ru) < tol
    assert _rel(mol.interior(out["v"].cpu().numpy(), og), rv) < tol


def test_etdrk4_coefficients_vs_phi(cuda):
    # the contour coefficients agree with the closed phi forms for |z| >> 1
    lam = -np.linspace(50.0, 400.0, 8)
    E, E2, Q, f1, f2, f3 = OE.etdrk4_coeffs(lam, 1.0)
    p1, p2, p3 = OE.phi_functions(lam)
    h1, _, _ = OE.phi_functions(lam / 2)
    np.testing.assert_allclose(Q, 0.5 * h1, rtol=1e-10)
    np.testing.assert_allclose(f1, p1 - 3 * p2 + 4 * p3, rtol=1e-9)
    np.testing.assert_allclose(f2, p2 - 2 * p3, rtol=1e-9)  # 2 f2 = b2 = 2 phi2 - 4 phi3
    np.testing.assert_allclose(f3, -p2 + 4 * p3, rtol=1e-9)


def test_etdrk4_fourth_order(cuda):
    # tests/test_fft_operators.py:561-617 style: error vs a fine reference drops ~16x per halving
    import moljax_gb300 as M
    n, L = 32, 2.5
    grid = M.Grid2D(n, n, 0.0, L, 0.0, L)
    model = M.create_gray_scott_model(grid, 2e-3, 1e-3, 0.035, 0.065)
    og = mol.Grid2D(n, n, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 3)
    ym = {k: torch.tensor(v, device=cuda) for k, v in y0.items()}
    ref = M.etdrk4_gray_scott(model, ym, 0.125, 64)["u"].cpu().numpy()
    errs = []
    for dt, n_st in ((2.0, 4), (1.0, 8)):
        errs.append(np.linalg.norm(M.etdrk4_gray_scott(model, ym, dt, n_st)["u"].cpu().numpy() - ref))
    assert errs[0] / errs[1] > 8.0


@pytest.mark.parametrize("ny,nx", [(4096, 16), (16, 4096)])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_etdrk4_maximum_extent(cuda, ny, nx, dtype):
    # 4096-point transforms along each axis (the widest column tiles and the 256-thread rows)
    import moljax_gb300 as M
    L = 2.5
    grid = M.Grid2D(nx, ny, 0.0, L, 0.0, L)
    model = M.create_gray_scott_model(grid, 2e-5, 1e-5, 0.035, 0.065, dtype=dtype)
    og = mol.Grid2D(nx, ny, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 23)
    ym = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
    out = M.etdrk4_gray_scott(model, ym, 0.5, 6)
    lam = mol.fd_symbol_2d(ny, nx, og.dy, og.dx)
    ru, rv = OE.etdrk4_gray_scott(mol.interior(y0["u"], og), mol.interior(y0["v"], og), lam,
                                  2e-5, 1e-5, 0.035, 0.065, 0.5, 6, 2.0)
    tol = 1e-11 if dtype == torch.float64 else 3e-6
    assert _rel(mol.interior(out["u"].cpu().numpy(), og), ru) < tol
    assert _rel(mol.interior(out["v"].cpu().numpy(), og), rv) < tol
