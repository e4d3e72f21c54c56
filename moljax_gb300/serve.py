"""Continuous-batching solve server for a mixed stream of PDE requests (one GPU).

Requests arrive over time (Poisson).  The server:

* admits a request once it has arrived and its device memory fits the free-HBM
  budget (workspace and state are reserved at admission, released at completion);
* batches tubular-reactor requests continuously: every reactor request admitted
  while a batch runs joins the next batch, and each batch is ONE launch of the
  batched reactor kernel (uneven sizes, one CTA per solve);
* runs Gray-Scott IMEX-Strang requests as independent adaptive solves on
  per-slot CUDA streams from worker threads (the native calls release the GIL),
  so several solves and reactor batches overlap on the device;
* records arrival, start and completion of every request and reports
  p50/p99 time-to-solution, solves/s and grid-point-steps/s.

``run_plain`` is the one-solve-at-a-time comparator (FIFO, FP64 by default).
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
_models: Dict[tuple, tuple] = {}
_lock = threading.Lock()


def _gs_setup(n, F, k, dtype, device):
    import moljax_gb300 as M
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, DU, DV, F, k, dtype, device)
    return M, grid, model, cache, diff


def solve_gs(req: Request, dtype=torch.float32, precision="mixed", device="cuda"):
    """One adaptive IMEX-Strang solve of a Gray-Scott request (rtol 1e-5, atol 1e-7)."""
    from moljax_gb300.workloads import gray_scott_initial_condition
    M, grid, model, cache, diff = _gs_setup(req.n, req.params["F"], req.params["k"], dtype, device)
    y0 = gray_scott_initial_condition(grid, 1000 + req.rid, dtype, device)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, y0, 0.0, req.params["t_end"], 1.0, cache, diff,
                                  pid_params=pid, max_steps=20000, save_every=100,
                                  save_y_history=False, precision=precision)
    out = torch.stack([r.y_final["u"], r.y_final["v"]])
    return out, float(req.n * req.n * r.n_accepted), {"accepted": r.n_accepted,
                                                      "rejected": r.n_rejected, "status": r.status}


def reactor_case(req: Request):
    from moljax_gb300.core import reactor as R
    dt, ns = R.served_dt(req.n)
    return R.ReactorCase(req.n, req.params["Pe"], req.params["Da"], dt, ns, R.DANCKWERTS, 0.0)


def request_bytes(req: Request, dtype=torch.float32, precision="mixed") -> int:
    """Device bytes reserved while a request is in flight."""
    from moljax_gb300 import _native as N
    es = 4 if dtype == torch.float32 else 8
    if req.kind == "reactor":
        return req.n * es + 256
    n = req.n
    if precision == "mixed":
        ws = N.lib().mjx_imex2d_mixed_ws_bytes(n, n, 2)
    else:
        ws = N.lib().mjx_imex2d_ws_bytes(n, n, 2, 0 if es == 4 else 1)
    return int(ws + 6 * (n + 2) ** 2 * es)


# ------------------------------------------------------------------ server
class Server:
    def __init__(self, device=None, slots: int = 8, hbm_budget: Optional[int] = None,
                 dtype=torch.float32, precision: str = "mixed"):
        self.device = torch.device(device or "cuda")
        self.slots = slots
        self.dtype = dtype
        self.precision = precision
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(0.5 * free)
        self.budget = int(hbm_budget)
        self.reserved = 0
        self.cv = threading.Condition()
        self.done: List[Completion] = []
        self.max_reserved = 0
        self.batches = 0

    def _reserve(self, b):
        if self.reserved + b > self.budget and self.reserved > 0:
            return False
        self.reserved += b
        self.max_reserved = max(self.max_reserved, self.reserved)
        return True

    def _release(self, b):
        with self.cv:
            self.reserved -= b
            self.cv.notify_all()

    def run(self, requests: List[Request], realtime: bool = True) -> List[Completion]:
        torch.cuda.set_device(self.device)
        # warm plans and kernels for every grid size in the mix (outside the clock)
        for n in sorted({r.n for r in requests if r.kind == "gs"}):
            _gs_setup(n, 0.035, 0.065, self.dtype, self.device)
        pending = sorted(requests, key=lambda r: r.arrival)
        reactor_q: List[tuple] = []
        pool = ThreadPoolExecutor(max_workers=self.slots)
        streams = [torch.cuda.Stream(self.device) for _ in range(self.slots)]
        free_streams = list(range(self.slots))
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0  # noqa: E731
        reactor_busy = [False]
        reactor_stream = torch.cuda.Stream(self.device)
        outstanding = [0]

        def gs_job(req, sidx, nbytes, start):
            with torch.cuda.device(self.device), torch.cuda.stream(streams[sidx]):
                out, pts, info = solve_gs(req, self.dtype, self.precision, self.device)
                torch.cuda.current_stream().synchronize()
            end = now()
            with self.cv:
                self.done.append(Completion(req.rid, "gs", req.arrival, start, end, out, pts, info))
                free_streams.append(sidx)
                self.reserved -= nbytes
                outstanding[0] -= 1
                self.cv.notify_all()

        def reactor_job(batch):
            from moljax_gb300.core import reactor as R
            start = now()
            with torch.cuda.device(self.device), torch.cuda.stream(reactor_stream):
                cases = [reactor_case(r) for r, _ in batch]
                outs = R.solve_batch(cases, self.dtype, self.device, reactor_stream.cuda_stream)
                reactor_stream.synchronize()
            end = now()
            with self.cv:
                for (req, nb), o, c in zip(batch, outs, cases):
                    self.done.append(Completion(req.rid, "reactor", req.arrival, start, end, o,
                                                float(c.n * c.n_steps), {"batch": len(batch)}))
                    self.reserved -= nb
                outstanding[0] -= len(batch)
                reactor_busy[0] = False
                self.batches += 1
                self.cv.notify_all()

        i = 0
        with self.cv:
            while i < len(pending) or outstanding[0] > 0 or reactor_q:
                t = now()
                # admit arrived requests while memory allows
                while i < len(pending) and (pending[i].arrival <= t or not realtime):
                    req = pending[i]
                    nb = request_bytes(req, self.dtype, self.precision)
                    if req.kind == "gs" and not free_streams:
                        break
                    if not self._reserve(nb):
                        break
                    outstanding[0] += 1
                    i += 1
                    if req.kind == "reactor":
                        reactor_q.append((req, nb))
                    else:
                        sidx = free_streams.pop()
                        pool.submit(gs_job, req, sidx, nb, t)
                # continuous batching: everything queued goes into the next launch
                if reactor_q and not reactor_busy[0]:
                    batch, reactor_q = reactor_q, []
                    reactor_busy[0] = True
                    pool.submit(reactor_job, batch)
                nxt = pending[i].arrival - now() if i < len(pending) else None
                timeout = max(0.0, nxt) if (nxt is not None and realtime) else 0.05
                self.cv.wait(timeout=min(timeout, 0.05))
        pool.shutdown(wait=True)
        self.makespan = now()
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
            o, pts, info = solve_gs(req, dtype, prec, dev)
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
