"""Native DST-I and the Dirichlet spectral solvers vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import dst as OD

pytestmark = pytest.mark.gpu

# direct FFT lengths (2(N+1) a power of two) and Bluestein lengths
SIZES = [1, 2, 3, 7, 31, 32, 64, 100, 127, 1000, 1023, 2047]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_dst_matches_oracle(cuda, n, dtype):
    import moljax_gb300 as M
    rng = np.random.default_rng(n)
    for shape in [(n,), (3, n), (2, 5, n)]:  # odd and even row counts
        x = rng.standard_normal(shape)
        X = M.dst_I_fast(torch.tensor(x, dtype=dtype, device=cuda)).cpu().numpy()
        ref = OD.dst_I_fast(x)
        assert X.shape == shape
        assert _rel(X, ref) < (1e-12 if dtype == torch.float64 else 2e-5), (shape, _rel(X, ref))
        back = M.idst_I_fast(torch.tensor(ref, dtype=dtype, device=cuda)).cpu().numpy()
        assert _rel(back, x) < (1e-12 if dtype == torch.float64 else 2e-5)


def test_reference_known_answers(cuda):
    # tests/test_fft_nonperiodic.py:24-46
    import moljax_gb300 as M
    N = 32
    x = torch.sin(torch.pi * torch.arange(1, N + 1, dtype=torch.float64) / (N + 1)).to(cuda)
    torch.testing.assert_close(M.idst_I_fast(M.dst_I_fast(x)), x, rtol=1e-10, atol=0)
    N = 64
    f = torch.sin(torch.pi * torch.arange(1, N + 1, dtype=torch.float64) / (N + 1)).to(cuda)
    F = M.dst_I_fast(f)
    assert abs(float(F[0])) > 0.9 * float(torch.linalg.norm(F))


@pytest.mark.parametrize("n", [31, 50, 255])
def test_dirichlet_solvers_vs_oracle(cuda, n):
    import moljax_gb300 as M
    rng = np.random.default_rng(7)
    dx, dt, D = 1.0 / (n + 1), 0.01, 0.5
    rhs = rng.standard_normal((4, n))
    lam = OD.laplacian_symbol_dirichlet(n, dx)
    cache = M.create_nonperiodic_fft_cache(n, dx, device=cuda)
    np.testing.assert_allclose(cache.laplacian_symbol.cpu().numpy(), lam, rtol=1e-14)
    r = torch.tensor(rhs, device=cuda)
    h = M.solve_helmholtz_dirichlet(r, cache.laplacian_symbol, dt, D).cpu().numpy()
    assert _rel(h, OD.solve_helmholtz_dirichlet(rhs, lam, dt, D)) < 1e-12
    p = M.solve_poisson_dirichlet(r, cache.laplacian_symbol).cpu().numpy()
    assert _rel(p, OD.solve_poisson_dirichlet(rhs, lam)) < 1e-12
    Nu = rng.standard_normal((4, n))
    e = M.etd1_dirichlet(r, torch.tensor(Nu, device=cuda), D * cache.laplacian_symbol, dt).cpu().numpy()
    assert _rel(e, OD.etd1_dirichlet(rhs, Nu, D * lam, dt)) < 1e-12


def test_unsupported_length_raises(cuda):
    import moljax_gb300 as M
    with pytest.raises(ValueError):
        M.dst_I_fast(torch.zeros(1500, dtype=torch.float64, device=cuda))


DCT_SIZES = [1, 2, 3, 5, 32, 64, 100, 1000, 1024, 2048]


@pytest.mark.parametrize("n", DCT_SIZES)
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_dct_matches_oracle(cuda, n, dtype):
    from moljax_gb300.core import fft_nonperiodic as F
    rng = np.random.default_rng(n + 7)
    for shape in [(n,), (3, n), (2, 5, n)]:
        x = rng.standard_normal(shape)
        X = F.dct(torch.tensor(x, dtype=dtype, device=cuda)).cpu().numpy()
        ref = OD.dct2_ortho(x)
        tol = 1e-12 if dtype == torch.float64 else 2e-5
        assert _rel(X, ref) < tol, (shape, _rel(X, ref))
        back = F.idct(torch.tensor(ref, dtype=dtype, device=cuda)).cpu().numpy()
        assert _rel(back, x) < tol


@pytest.mark.parametrize("n", [32, 50, 256])
def test_neumann_solvers_vs_oracle(cuda, n):
    from moljax_gb300.core import fft_nonperiodic as F
    import moljax_gb300 as M
    rng = np.random.default_rng(11)
    dx, dt, D = 1.0 / n, 0.01, 0.5
    rhs = rng.standard_normal((4, n))
    rhs_c = rhs - rhs.mean(axis=-1, keepdims=True)
    cache = M.create_nonperiodic_fft_cache(n, dx, "neumann", device=cuda)
    lam = OD.laplacian_symbol_neumann(n, dx)
    np.testing.assert_allclose(cache.laplacian_symbol.cpu().numpy(), lam, rtol=1e-14, atol=1e-300)
    r = torch.tensor(rhs, device=cuda)
    h = F.solve_helmholtz_neumann(r, cache.laplacian_symbol, dt, D).cpu().numpy()
    assert _rel(h, OD.solve_helmholtz_neumann(rhs, lam, dt, D)) < 1e-12
    p = F.solve_poisson_neumann(torch.tensor(rhs_c, device=cuda), cache.laplacian_symbol).cpu().numpy()
    assert _rel(p, OD.solve_poisson_neumann(rhs_c, lam)) < 1e-12
    Nu = rng.standard_normal((4, n))
    e = F.etd1_neumann(r, torch.tensor(Nu, device=cuda), D * cache.laplacian_symbol, dt).cpu().numpy()
    assert _rel(e, OD.etd1_neumann(rhs, Nu, D * lam, dt)) < 1e-12
    assert not F.check_compatibility_neumann(torch.ones(32, device=cuda))
    assert F.check_compatibility_neumann(F.project_to_compatible(torch.ones(32, dtype=torch.float64, device=cuda)))
