"""The autotuner on the GPU: every candidate radix schedule (and threads per sequence)
of a mixed-radix length computes the same transform (against NumPy), the tuner installs
one of its candidates, and every stencil tile height gives bit-identical stage output."""

import numpy as np
import pytest
import torch

from oracle.mol import fd_symbol_1d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [48, 100, 80, 96, 375])
def test_every_schedule_matches_numpy(cuda, n):
    import moljax_gb300 as M
    from moljax_gb300 import _native as N
    from moljax_gb300.core import autotune as AT
    from moljax_gb300.core.fft_solvers import GeneralSpectralPlan
    ny, nx = 64, n
    dy, dx = 0.9 / ny, 1.1 / nx
    plan = GeneralSpectralPlan(ny, nx, dy, dx, "fd", torch.float64, cuda)
    rng = np.random.default_rng(n)
    u = rng.standard_normal((ny, nx))
    lam = fd_symbol_1d(ny, dy)[:, None] + fd_symbol_1d(nx, dx)[None, :]
    ref = np.real(np.fft.ifft2(np.fft.fft2(u) / (1 - 0.01 * 0.3 * lam)))
    ut = torch.tensor(u, device=cuda)
    cands = AT.dft_schedule_candidates(n)
    assert cands
    try:
        for sched in cands:
            for tp in (n // 4, n // 8, max(1, n // 16)):
                AT.set_dft_schedule(n, torch.float64, sched, min(tp, 256))
                got = plan.apply(ut, [0.3], 0.01, N.MULT_HELMHOLTZ).cpu().numpy()
                err = float(np.max(np.abs(got - ref)))
                assert err < 1e-12, (sched, tp, err)
        res = AT.autotune_dft(n, torch.float64, cuda, nrows=ny)
        assert len(res.times_ms) == len(res.candidates) and 0 <= res.best < len(res.candidates)
        assert all(t > 0 for t in res.times_ms)
        sched, tp = res.choice
        assert (tuple(sched), tp) == tuple(res.candidates[res.best])
        assert AT.dft_schedule(n, torch.float64) == (tuple(sched), tp)
        got = plan.apply(ut, [0.3], 0.01, N.MULT_HELMHOLTZ).cpu().numpy()
        assert float(np.max(np.abs(got - ref))) < 1e-12
    finally:
        AT.set_dft_schedule(n, torch.float64, ())
    assert M.autotune is AT


def test_fp32_schedules_and_3d_plan(cuda):
    import moljax_gb300 as M
    from moljax_gb300 import _native as N
    from moljax_gb300.core import autotune as AT
    from moljax_gb300.core.fft_solvers import GeneralSpectralPlan
    n = 60
    plan = GeneralSpectralPlan(n, n, 1.0 / n, 1.0 / n, "fd", torch.float32, cuda)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((n, n))
    lam = fd_symbol_1d(n, 1.0 / n)[:, None] + fd_symbol_1d(n, 1.0 / n)[None, :]
    ref = np.real(np.fft.ifft2(np.exp(1e-4 * lam) * np.fft.fft2(u)))
    ut = torch.tensor(u, dtype=torch.float32, device=cuda)
    try:
        for sched in AT.dft_schedule_candidates(n):
            AT.set_dft_schedule(n, torch.float32, sched, 0)
            got = plan.apply(ut, [1.0], 1e-4, N.MULT_EXP).cpu().double().numpy()
            assert float(np.max(np.abs(got - ref))) < 2e-5, sched
    finally:
        AT.set_dft_schedule(n, torch.float32, ())
    # a 3D general plan tunes its lengths on creation and still matches the 3D oracle
    from oracle import fftcn as OF
    u3 = OF.node_grid_ic_3d(48)
    c3 = M.fft_cn_step_3d(torch.tensor(u3, device=cuda), 0.1, 1 / 48, 1e-3, 4).cpu().numpy()
    assert float(np.max(np.abs(c3 - OF.fft_cn_3d(u3, 0.1, 1 / 48, 1e-3, 4)))) < 1e-13
    assert AT.dft_schedule(48, torch.float64)[0]


@pytest.mark.parametrize("shape", [(96, 160), (37, 70), (70, 300)])
def test_stencil_tile_heights_bit_identical(cuda, shape):
    import moljax_gb300 as M
    from moljax_gb300.core import autotune as AT
    from moljax_gb300.core.bc import BCType
    ny, nx = shape
    grid = M.Grid2D(nx, ny, 0.0, 1.0, 0.0, 1.0)
    model = M.create_advection_diffusion_model(grid, ("c1", "c2"), 0.01, 0.6, -0.3, BCType(1), True,
                                               dtype=torch.float32)
    rng = np.random.default_rng(ny)
    y = {k: torch.tensor(rng.uniform(0, 1, (ny + 2, nx + 2)), dtype=torch.float32, device=cuda)
         for k in ("c1", "c2")}
    try:
        outs = []
        for rows in (2, 4, 8, 16, 32, 64):  # 64: the TMA-staged form where nx % 4 == 0
            AT.set_stencil_rows(ny, nx, 2, torch.float32, rows)
            F = model.rhs(y)
            outs.append(torch.stack([F["c1"], F["c2"]]).cpu())
        for o in outs[1:]:
            assert torch.equal(o, outs[0])
        res = AT.autotune_stencil(model, torch.float32)
        tma = nx % 4 == 0
        assert res.choice[0] in ((2, 4, 8, 16, 32, 64) if tma else (2, 4, 8, 16, 32))
        assert len(res.times_ms) == (6 if tma else 5)
        assert AT.stencil_rows(ny, nx, 2, torch.float32) == res.choice[0]
        F = model.rhs(y)
        assert torch.equal(torch.stack([F["c1"], F["c2"]]).cpu(), outs[0])
    finally:
        AT.set_stencil_rows(ny, nx, 2, torch.float32, 0)
