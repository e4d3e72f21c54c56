"""Continuous-batching solve server for a mixed stream of PDE requests (one GPU).

Requests arrive over time (Poisson).  The server:

* admits a request once it has arrived and its device memory fits the free-HBM
  budget (the bytes its solve allocates are reserved at admission and released
  at completion);
* runs every Gray-Scott IMEX-Strang request in one batch engine
  (``GrayScottBatch``): each attempt stage is one kernel launch over all solves
  in flight, each with its own dt, controller, accept mask and status.  A
  request that arrives while an epoch runs raises the engine's stop flag when a
  slot is free, so it joins at the next attempt boundary; every epoch also ends
  when a solve finishes, so results leave as soon as they are done;
* batches tubular-reactor requests continuously: every reactor request admitted
  while a batch runs joins the next batch, and each batch is ONE launch of the
  batched reactor kernel (uneven sizes, one CTA per solve);
* records arrival, start and completion of every request and reports
  p50/p99 time-to-solution, solves/s and grid-point-steps/s.

The two engines run in their own threads on their own CUDA streams, so reactor
batches overlap the Gray-Scott attempts on the device.  ``run_plain`` is the
one-solve-at-a-time comparator (FIFO, FP64 by default).
"""

from __future__ import annotations

import math
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

L_BOX = 2.5
DU, DV = 2e-5, 1e-5


@dataclass
class Request:
    rid: int
    kind: str                 # "reactor" | "gs"
    arrival: float            # seconds after the start of the run
    n: int                    # reactor points or GS grid side
    params: Dict[str, float] = field(default_factory=dict)


@dataclass
class Completion:
    rid: int
    kind: str
    arrival: float
    start: float
    end: float
    output: torch.Tensor
    pt_steps: float
    info: Dict[str, float] = field(default_factory=dict)

    @property
    def latency(self):
        return self.end - self.arrival


def make_mix(n_requests: int = 4096, rate: float = 2000.0, seed: int = 5,
             reactor_frac: float = 0.6, gs_sizes=(64, 128, 256, 512)) -> List[Request]:
    """The served mix: Poisson arrivals; 60 % reactor (Danckwerts CN, n log-uniform in
    [64, 4096], Pe~U[10,200], Da~U[0.5,5], c0 = 0, t_final = 5); 40 % Gray-Scott
    IMEX-Strang (grid side in gs_sizes, F~U[0.02,0.06], k~U[0.05,0.07], t_end = 100)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n_requests))
    out = []
    for i in range(n_requests):
        if rng.uniform() < reactor_frac:
            n = int(round(math.exp(rng.uniform(math.log(64), math.log(4096)))))
            out.append(Request(i, "reactor", float(t[i]), n,
                               {"Pe": float(rng.uniform(10, 200)), "Da": float(rng.uniform(0.5, 5.0))}))
        else:
            n = int(gs_sizes[rng.integers(len(gs_sizes))])
            out.append(Request(i, "gs", float(t[i]), n,
                               {"F": float(rng.uniform(0.02, 0.06)), "k": float(rng.uniform(0.05, 0.07)),
                                "t_end": 100.0}))
    return out


# ------------------------------------------------------------------ per-request work
def _gs_setup(n, F, k, dtype, device):
    import moljax_gb300 as M
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, DU, DV, F, k, dtype, device)
    return M, grid, model, cache, diff


def gs_initial_state(req: Request, dtype=torch.float32, device="cuda"):
    """The request's initial state: the seeded Gray-Scott square-plus-noise state
    (examples/gray_scott_2d.py:42-73, seed 1000 + rid), a padded (u, v) StateDict."""
    import moljax_gb300 as M
    from moljax_gb300.workloads import gray_scott_initial_condition
    grid = M.Grid2D(req.n, req.n, 0.0, L_BOX, 0.0, L_BOX)
    return gray_scott_initial_condition(grid, 1000 + req.rid, dtype, device)


def solve_gs(req: Request, dtype=torch.float32, precision="mixed", device="cuda"):
    """One adaptive IMEX-Strang solve of a Gray-Scott request alone (rtol 1e-5, atol 1e-7);
    returns the interior (2, n, n) final state, the grid-point-steps and the counts."""
    M, grid, model, cache, diff = _gs_setup(req.n, req.params["F"], req.params["k"], dtype, device)
    y0 = gs_initial_state(req, dtype, device)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, y0, 0.0, req.params["t_end"], 1.0, cache, diff,
                                  pid_params=pid, max_steps=20000, save_every=100,
                                  save_y_history=False, precision=precision)
    out = M.stencil.unpad(torch.stack([r.y_final["u"], r.y_final["v"]]), grid)
    return out, float(req.n * req.n * r.n_accepted), {"accepted": r.n_accepted,
                                                      "rejected": r.n_rejected, "status": r.status}


def gs_problem(req: Request, y0):
    """The batch-engine problem of a Gray-Scott request (the solve_gs settings)."""
    import moljax_gb300 as M
    grid = M.Grid2D(req.n, req.n, 0.0, L_BOX, 0.0, L_BOX)
    return M.GrayScottProblem(grid, DU, DV, req.params["F"], req.params["k"], y0, 0.0, req.params["t_end"], 1.0,
                              pid=M.PIDParams(atol=1e-7, rtol=1e-5), max_steps=20000, save_every=100)


def reactor_case(req: Request):
    from moljax_gb300.core import reactor as R
    dt, ns = R.served_dt(req.n)
    # the CN step size of benchmark_method_comparison.py:216 needs the fully implicit CN
    return R.ReactorCase(req.n, req.params["Pe"], req.params["Da"], dt, ns, R.DANCKWERTS_CN, 0.0)


def request_bytes(req: Request, dtype=torch.float32) -> int:
    """Device bytes a request allocates while in flight: for Gray-Scott the batch
    engine's per-solve workspace (spectral state, plans, partials, t/dt history) plus
    its initial and final states; for the reactor its output profile and instance entry."""
    from moljax_gb300.core.batch import GrayScottBatch
    es = 4 if dtype == torch.float32 else 8
    if req.kind == "reactor":
        return req.n * es + 64
    n = req.n
    return GrayScottBatch.instance_bytes(n, n, 20000, 100) + 2 * (n + 2) ** 2 * es + 2 * n * n * es


# ------------------------------------------------------------------ server
class Server:
    """Serves a list of requests (see the module docstring).  ``slots`` is the number
    of Gray-Scott solves the batch engine holds at once; ``hbm_budget`` bounds the
    bytes reserved by requests in flight (default: half of the free device memory)."""

    def __init__(self, device=None, slots: int = 64, hbm_budget: Optional[int] = None,
                 dtype=torch.float32, stall_s: float = 120.0):
        self.device = torch.device(device or "cuda")
        self.stall_s = float(stall_s)  # no completion for this long raises (a stuck run)
        self.slots = int(slots)
        self.dtype = dtype
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(0.5 * free)
        self.budget = int(hbm_budget)
        self.reserved = 0
        self.cv = threading.Condition()
        self.done: List[Completion] = []
        self.max_reserved = 0
        self.batches = 0
        self.epochs = 0

    def _reserve(self, b):
        if self.reserved + b > self.budget and self.reserved > 0:
            return False
        self.reserved += b
        self.max_reserved = max(self.max_reserved, self.reserved)
        return True

    def run(self, requests: List[Request], realtime: bool = True) -> List[Completion]:
        from moljax_gb300.core import reactor as R
        from moljax_gb300.core.batch import GrayScottBatch
        torch.cuda.set_device(self.device)
        # the engine, its kernels and the host initial states are set up outside the clock
        eng = GrayScottBatch(self.device, max_instances=self.slots,
                             max_work=self.slots * 388)  # 388: work items of a 512^2 solve
        y0s = {r.rid: gs_initial_state(r, self.dtype, "cpu").copy() for r in requests if r.kind == "gs"}
        y0s = {k: {f: t.pin_memory() for f, t in v.items()} for k, v in y0s.items()}
        pending = sorted(requests, key=lambda r: r.arrival)
        gs_q: List[Request] = []
        reactor_q: List[tuple] = []
        gs_stream = torch.cuda.Stream(self.device)
        reactor_stream = torch.cuda.Stream(self.device)
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        state = {"closing": False, "reactor_busy": False, "live": {}, "error": None}

        def gs_loop():
            live = state["live"]
            try:
                with torch.cuda.device(self.device), torch.cuda.stream(gs_stream):
                    while True:
                        admit = []
                        with self.cv:
                            while gs_q and eng.fits(gs_q[0].n, gs_q[0].n) and len(live) + len(admit) < self.slots:
                                nb = request_bytes(gs_q[0], self.dtype)
                                if not self._reserve(nb):
                                    break
                                admit.append((gs_q.pop(0), nb))
                            if state["error"] is not None:
                                return
                            if not admit and not live:
                                if state["closing"] and not gs_q:
                                    return
                                self.cv.wait(0.02)
                                continue
                        for req, nb in admit:
                            y0 = {f: t.to(self.device, non_blocking=True) for f, t in y0s[req.rid].items()}
                            slot = eng.admit(gs_problem(req, y0))
                            live[slot] = (req, nb, now())
                        eng.request_stop(False)
                        eng.run(stop_after_finished=1)
                        self.epochs += 1
                        for slot in eng.finished():
                            out, r = eng.retire(slot, self.dtype)
                            req, nb, start = live.pop(slot)
                            end = now()
                            with self.cv:
                                self.done.append(Completion(req.rid, "gs", req.arrival, start, end, out,
                                                            float(req.n * req.n * r.n_accepted),
                                                            {"accepted": r.n_accepted, "rejected": r.n_rejected,
                                                             "status": r.status}))
                                self.reserved -= nb
                                self.cv.notify_all()
            except Exception as e:  # noqa: BLE001 - reported by run()
                state["error"] = e
                with self.cv:
                    self.cv.notify_all()

        def reactor_job(batch):
            start = now()
            try:
                with torch.cuda.device(self.device), torch.cuda.stream(reactor_stream):
                    cases = [reactor_case(r) for r, _ in batch]
                    outs = R.solve_batch(cases, self.dtype, self.device, reactor_stream.cuda_stream)
                    reactor_stream.synchronize()
            except Exception as e:  # noqa: BLE001 - reported by run()
                with self.cv:
                    state["error"] = e
                    self.cv.notify_all()
                return
            end = now()
            with self.cv:
                for (req, nb), o, c in zip(batch, outs, cases):
                    self.done.append(Completion(req.rid, "reactor", req.arrival, start, end, o,
                                                float(c.n * c.n_steps), {"batch": len(batch)}))
                    self.reserved -= nb
                state["reactor_busy"] = False
                self.batches += 1
                self.cv.notify_all()

        pool = ThreadPoolExecutor(max_workers=2)
        gs_thread = threading.Thread(target=gs_loop, daemon=True)
        gs_thread.start()
        i = 0
        n_total = len(pending)
        last_progress, last_done = now(), 0
        with self.cv:
            while len(self.done) < n_total and state["error"] is None:
                t = now()
                if len(self.done) != last_done:
                    last_progress, last_done = t, len(self.done)
                elif t - last_progress > self.stall_s:
                    state["error"] = RuntimeError(
                        f"no request completed for {self.stall_s:.0f} s: {len(self.done)}/{n_total} done, "
                        f"{len(gs_q)} Gray-Scott queued, {len(state['live'])} in the engine, "
                        f"{len(reactor_q)} reactor queued, reserved {self.reserved} of {self.budget} bytes")
                    eng.request_stop(True)
                    break
                # arrivals: reactor requests reserve their bytes here; Gray-Scott requests
                # queue for the engine, which reserves when it admits them
                while i < len(pending) and (pending[i].arrival <= t or not realtime):
                    req = pending[i]
                    if req.kind == "gs":
                        gs_q.append(req)
                        i += 1
                        if len(state["live"]) < self.slots:
                            eng.request_stop(True)  # join at the next attempt boundary
                        continue
                    nb = request_bytes(req, self.dtype)
                    if not self._reserve(nb):
                        break
                    reactor_q.append((req, nb))
                    i += 1
                # continuous batching: every queued reactor request goes into the next launch
                if reactor_q and not state["reactor_busy"]:
                    batch, reactor_q = reactor_q, []
                    state["reactor_busy"] = True
                    pool.submit(reactor_job, batch)
                self.cv.notify_all()
                nxt = pending[i].arrival - now() if i < len(pending) else None
                timeout = max(0.0, nxt) if (nxt is not None and realtime) else 0.02
                self.cv.wait(timeout=min(timeout, 0.02))
            state["closing"] = True
            self.cv.notify_all()
        gs_thread.join(timeout=None if state["error"] is None else 60.0)
        pool.shutdown(wait=True)
        self.makespan = now()
        eng.close()
        if state["error"] is not None:
            raise state["error"]
        return sorted(self.done, key=lambda c: c.rid)


def run_plain(requests: List[Request], dtype=torch.float64, device="cuda",
              realtime: bool = True) -> List[Completion]:
    """One solve at a time, FIFO (the plain comparator); FP64 by default."""
    from moljax_gb300.core import reactor as R
    dev = torch.device(device)
    for n in sorted({r.n for r in requests if r.kind == "gs"}):
        _gs_setup(n, 0.035, 0.065, dtype, dev)
    prec = "fp64" if dtype == torch.float64 else "fp32"
    t0 = time.perf_counter()
    out = []
    for req in sorted(requests, key=lambda r: r.arrival):
        t = time.perf_counter() - t0
        if realtime and req.arrival > t:
            time.sleep(req.arrival - t)
        start = time.perf_counter() - t0
        if req.kind == "gs":
            o, pts, info = solve_gs(req, dtype, prec, dev)  # interior (2, n, n)
        else:
            c = reactor_case(req)
            o = R.solve_batch([c], dtype, dev)[0]
            pts, info = float(c.n * c.n_steps), {}
        torch.cuda.synchronize(dev)
        end = time.perf_counter() - t0
        out.append(Completion(req.rid, req.kind, req.arrival, start, end, o, pts, info))
    return out


def summarize(done: List[Completion], makespan: float) -> Dict[str, float]:
    lat = np.array([c.latency for c in done])
    res = {"n": len(done), "makespan_s": makespan, "solves_per_s": len(done) / makespan,
           "pt_steps_per_s": float(sum(c.pt_steps for c in done)) / makespan,
           "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99))}
    for kind in ("reactor", "gs"):
        lk = np.array([c.latency for c in done if c.kind == kind])
        if len(lk):
            res[f"{kind}_p50_s"] = float(np.percentile(lk, 50))
            res[f"{kind}_p99_s"] = float(np.percentile(lk, 99))
    return res
