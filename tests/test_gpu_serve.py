"""Continuous-batching server: results alone == in the mix; admission under a tiny budget."""

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _small_mix(n=24):
    from moljax_gb300.serve import make_mix
    mix = make_mix(n, rate=400.0, seed=11, gs_sizes=(64, 128))
    for r in mix:
        if r.kind == "gs":
            r.params["t_end"] = 20.0
        else:
            r.n = min(r.n, 1024)
    return mix


def test_served_results_equal_alone(cuda):
    from moljax_gb300.serve import Server, solve_gs, reactor_case
    from moljax_gb300.core import reactor as R
    mix = _small_mix()
    done = Server(cuda, slots=4).run(mix)
    assert len(done) == len(mix)
    by_id = {c.rid: c for c in done}
    for req in mix[:10]:
        if req.kind == "gs":
            alone, _, _ = solve_gs(req, torch.float32, "mixed", cuda)
        else:
            alone = R.solve_batch([reactor_case(req)], torch.float32, cuda)[0]
        got = by_id[req.rid].output
        err = float(torch.linalg.norm(got.double() - alone.double()) / torch.linalg.norm(alone.double()))
        assert err < 1e-6, (req.kind, req.n, err)


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


def test_plain_comparator_matches_oracle_mix(cuda):
    from moljax_gb300.serve import run_plain, summarize
    mix = _small_mix(6)
    done = run_plain(mix, torch.float64, cuda, realtime=False)
    s = summarize(done, max(c.end for c in done))
    assert s["n"] == 6 and s["p99_s"] >= s["p50_s"] > 0
