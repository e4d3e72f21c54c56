"""Batched adaptive IMEX-Strang (mjx_gsbatch_*) vs the single-solve mixed path and the oracle.

Solves of different grid sizes, parameters and time spans share one engine;
each must take the same accept/reject sequence and reach the same state as
when it runs alone (bitwise: the engine's arithmetic for one solve does not
depend on the others), agree with the single-solve mixed-precision driver and
with the NumPy FP64 oracle (rel-L2 1e-6, equal step counts).
"""

import numpy as np
import pytest
import torch

from oracle import imex as OI
from oracle import mol

pytestmark = pytest.mark.gpu

L = 2.5
DU, DV = 2e-5, 1e-5


def _problem(ny, nx, F, k, t_end, seed, device, **kw):
    import moljax_gb300 as M
    grid = M.Grid2D(nx, ny, 0.0, L, 0.0, L)
    og = mol.Grid2D(nx, ny, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, seed)
    ym = {k_: torch.tensor(v, dtype=torch.float32, device=device) for k_, v in y0.items()}
    p = M.GrayScottProblem(grid, DU, DV, F, k, ym, 0.0, t_end, 1.0,
                           pid=M.PIDParams(atol=1e-7, rtol=1e-5), **kw)
    return p, og, y0


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


CASES = [(64, 64, 0.035, 0.065, 12.0, 1), (32, 32, 0.03, 0.06, 20.0, 2), (128, 128, 0.045, 0.062, 6.0, 3),
         (32, 128, 0.05, 0.065, 9.0, 4), (64, 16, 0.025, 0.055, 15.0, 5), (16, 16, 0.04, 0.06, 25.0, 6)]


def test_batch_matches_single_mixed_and_oracle(cuda):
    import moljax_gb300 as M
    probs = [_problem(*c, cuda, max_steps=4000, save_every=50) for c in CASES]
    res = M.adaptive_integrate_imex_batch([p for p, _, _ in probs], cuda)
    for (p, og, y0), (out, r), c in zip(probs, res, CASES):
        # the single-solve mixed driver
        model, cache, diff = M.create_gray_scott_periodic_fft(p.grid, DU, DV, p.F, p.k, torch.float32, cuda)
        rs = M.adaptive_integrate_imex(model, p.y0, 0.0, p.t_end, 1.0, cache, diff, pid_params=p.pid,
                                       max_steps=4000, save_every=50, save_y_history=False, precision="mixed")
        assert r.status == rs.status == 0, c
        assert (r.n_accepted, r.n_rejected) == (rs.n_accepted, rs.n_rejected), c
        assert r.t_final == pytest.approx(rs.t_final, abs=1e-12)
        for i, f in enumerate(("u", "v")):
            single = M.stencil.unpad(rs.y_final[f][None], p.grid)[0].cpu().numpy()
            assert _rel(out[i].cpu().numpy(), single) < 1e-6, (c, f)
        # the FP64 oracle
        om, lam, od = OI.gray_scott_periodic(og, DU, DV, p.F, p.k)
        ro = OI.adaptive_integrate_imex(om, y0, 0.0, p.t_end, 1.0, lam, od,
                                        pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=50,
                                        max_steps=4000, keep_history=False)
        assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected), c
        for i, f in enumerate(("u", "v")):
            assert _rel(out[i].cpu().numpy(), mol.interior(ro.y_final[f], og)) < 1e-6, (c, f)
        # t history written by the device controller (every 50th accepted step); dt follows
        # the error ratio, which the mixed form evaluates from FP32 transforms (~1e-5 relative)
        nh = r.n_steps
        assert nh == ro.n_steps
        np.testing.assert_allclose(r.t_history.numpy()[:nh], ro.t_history[:nh], rtol=1e-4)


def test_alone_equals_in_batch_with_continuous_admission(cuda):
    """Each solve gives bit-identical results alone and in a batch whose other members
    are admitted and retired while it runs."""
    import moljax_gb300 as M
    alone = {}
    for c in CASES[:4]:
        p, _, _ = _problem(*c, cuda)
        (out, r), = M.adaptive_integrate_imex_batch([p], cuda)
        alone[c] = (out.cpu(), r)
    eng = M.GrayScottBatch(cuda, max_instances=3)
    pending = list(CASES[:4]) * 2  # every case twice, admitted as slots free up
    got, live = [], {}
    while pending or live:
        while pending and eng.fits(pending[0][0], pending[0][1]):
            c = pending.pop(0)
            p, _, _ = _problem(*c, cuda)
            live[eng.admit(p)] = c
        eng.run(stop_after_finished=1)
        for s in eng.finished():
            out, r = eng.retire(s)
            got.append((live.pop(s), out.cpu(), r))
    assert len(got) == 8
    for c, out, r in got:
        a_out, a_r = alone[c]
        assert (r.n_accepted, r.n_rejected, r.status) == (a_r.n_accepted, a_r.n_rejected, a_r.status)
        assert torch.equal(out, a_out), c
    eng.close()


def test_batch_status_paths(cuda):
    """A solve that hits max_steps, one with a NaN in its state and a normal one, together."""
    import moljax_gb300 as M
    p1, _, _ = _problem(32, 32, 0.035, 0.065, 100.0, 7, cuda, max_steps=5)
    p2, _, _ = _problem(32, 32, 0.035, 0.065, 5.0, 8, cuda)
    p2.y0["u"][5, 7] = float("nan")
    p3, _, _ = _problem(64, 64, 0.035, 0.065, 3.0, 9, cuda)
    (o1, r1), (o2, r2), (o3, r3) = M.adaptive_integrate_imex_batch([p1, p2, p3], cuda)
    assert r1.status == M.StatusCode.MAX_STEPS_REACHED and r1.n_accepted == 5
    assert r2.status == M.StatusCode.NON_FINITE_VALUES
    assert r3.status == M.StatusCode.SUCCESS and r3.t_final == pytest.approx(3.0)


def test_batch_rejects_unsupported_sizes(cuda):
    import moljax_gb300 as M
    g = M.Grid2D(8, 8, 0.0, L, 0.0, L)
    p = M.GrayScottProblem(g, DU, DV, 0.035, 0.065, torch.zeros(2, 8, 8, device=cuda), 0.0, 1.0)
    eng = M.GrayScottBatch(cuda, max_instances=2)
    with pytest.raises(ValueError):
        eng.admit(p)
    eng.close()
