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
