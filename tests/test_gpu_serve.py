"""Continuous-batching server: results alone == in the mix; admission under a tiny
budget; the plain FP64 comparator against the oracle."""

import numpy as np
import pytest
import torch

from oracle import imex as OI
from oracle import mol
from oracle import reactor as OR

pytestmark = pytest.mark.gpu


def _small_mix(n=24, seed=11):
    from moljax_gb300.serve import make_mix
    mix = make_mix(n, rate=400.0, seed=seed, gs_sizes=(64, 128))
    for r in mix:
        if r.kind == "gs":
            r.params["t_end"] = 20.0
        else:
            r.n = min(r.n, 1024)
    return mix


def test_served_results_equal_alone(cuda):
    """Each Gray-Scott result of the served mix equals the same request solved alone in
    the batch engine (bitwise) and the single-solve mixed driver (rel-L2 1e-6); each
    reactor result equals its solve alone (bitwise)."""
    import moljax_gb300 as M
    from moljax_gb300.serve import Server, solve_gs, reactor_case, gs_problem, gs_initial_state
    from moljax_gb300.core import reactor as R
    mix = _small_mix()
    srv = Server(cuda, slots=4)
    done = srv.run(mix)
    assert len(done) == len(mix) and srv.epochs > 1
    by_id = {c.rid: c for c in done}
    for req in mix[:12]:
        got = by_id[req.rid].output
        if req.kind == "gs":
            (alone, r), = M.adaptive_integrate_imex_batch([gs_problem(req, gs_initial_state(req, torch.float32, cuda))],
                                                          cuda)
            assert torch.equal(got, alone), req.rid
            single, _, info = solve_gs(req, torch.float32, "mixed", cuda)
            assert info["accepted"] == r.n_accepted and info["rejected"] == r.n_rejected
            err = float(torch.linalg.norm(got.double() - single.double()) / torch.linalg.norm(single.double()))
            assert err < 1e-6, (req.n, err)
        else:
            alone = R.solve_batch([reactor_case(req)], torch.float32, cuda)[0]
            assert torch.equal(got, alone), req.rid


def test_admission_with_tiny_budget(cuda):
    from moljax_gb300.serve import Server, request_bytes
    mix = _small_mix(12)
    srv = Server(cuda, slots=4, hbm_budget=1)
    done = srv.run(mix, realtime=False)
    assert len(done) == len(mix)
    # with a 1-byte budget only one request is ever in flight
    assert srv.max_reserved <= max(request_bytes(r) for r in mix)
    starts = sorted((c.start, c.end) for c in done)
    for (s0, e0), (s1, e1) in zip(starts, starts[1:]):
        assert s1 >= e0 - 1e-3


def test_plain_comparator_matches_oracle(cuda):
    """The plain one-solve-at-a-time FP64 comparator reproduces the oracle: Gray-Scott
    adaptive IMEX-Strang (same step counts, rel-L2 1e-10) and the Danckwerts CN reactor."""
    from moljax_gb300.serve import run_plain, summarize, reactor_case, L_BOX, DU, DV
    mix = _small_mix(6, seed=3)
    done = run_plain(mix, torch.float64, cuda, realtime=False)
    s = summarize(done, max(c.end for c in done))
    assert s["n"] == 6 and s["p99_s"] >= s["p50_s"] > 0
    by_id = {c.rid: c for c in done}
    kinds = set()
    for req in mix:
        got = by_id[req.rid].output.cpu().numpy()
        kinds.add(req.kind)
        if req.kind == "gs":
            og = mol.Grid2D(req.n, req.n, 0, L_BOX, 0, L_BOX)
            from moljax_gb300.workloads import gray_scott_initial_condition
            import moljax_gb300 as M
            y0 = gray_scott_initial_condition(M.Grid2D(req.n, req.n, 0.0, L_BOX, 0.0, L_BOX), 1000 + req.rid,
                                              torch.float64, "cpu")
            y0 = {k: v.numpy() for k, v in y0.items()}
            om, lam, od = OI.gray_scott_periodic(og, DU, DV, req.params["F"], req.params["k"])
            ro = OI.adaptive_integrate_imex(om, y0, 0.0, req.params["t_end"], 1.0, lam, od,
                                            pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=100,
                                            max_steps=20000, keep_history=False)
            assert by_id[req.rid].info["accepted"] == ro.n_accepted
            assert by_id[req.rid].info["rejected"] == ro.n_rejected
            for i, f in enumerate(("u", "v")):
                ref = mol.interior(ro.y_final[f], og)
                assert float(np.linalg.norm(got[i] - ref) / np.linalg.norm(ref)) < 1e-10
        else:
            c = reactor_case(req)
            ref = OR.danckwerts_full_cn(c.n, c.Pe, c.Da, c.dt, c.n_steps, c.c_init)
            assert float(np.max(np.abs(got - ref))) < 1e-10
            assert np.all(np.isfinite(got)) and 0.0 < got[-1] < 1.0  # outlet below the inlet
    assert kinds == {"gs", "reactor"}
