"""Benchmark: adaptive IMEX-Strang Gray-Scott, 1024^2, t in (0, 2000).

One "step" is one full adaptive solve over t_span = (0, 2000) (step doubling,
PI control, accept/reject all on the device).  The metric is
grid-point-steps/s = interior points x accepted steps / time.  The default
precision is "mixed": float-float (FP32 pair) spectral state, FP32 transforms
of the reaction increments (rel-L2 vs the FP64 path is reported in the line).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --kernels-only [--reps R] [--graph]   # per-kernel CUDA-event times only
  python bench.py --workload etdrk4 --n 4096 [--etd-steps S] [--kernels-only] [--etd-method etd1|etd2]
  python bench.py --workload serve [--requests R]
  python bench.py --workload fft3d --n 512 [--etd-steps S] [--fp32]
  python bench.py --workload explicit --n 4096 [--etd-steps S]      (RK4 advection-diffusion)
  python bench.py --workload nk --n 512 [--etd-steps S]             (BDF2 Newton-Krylov)
  python bench.py --workload stencil --n 4096 [--fp32]               (stencil stage kernel roofline)
  python bench.py --workload gs256        (the reference's Gray-Scott method benchmark, 256^2 FP64)
  python bench.py --workload tubular      (the reference's 27-case penalty-RK4 reactor sweep, FP64)

Our arm prints one JSON line with the device-timed value, the end-to-end
number through the public API with host buffers, the live roofline of the
dominant kernel, the error against the FP64 path, the CPU baseline and SM
clocks.  ``--impl reference`` times the CPU restatement of the reference
algorithm (NumPy/SciPy FP64, all host threads) on a bounded sample of the same
workload.  The path does not shard: N > 1 runs N independent replicas (one per
rank).  ``--kernels-only`` launches each attempt kernel R times through the
per-kernel entry point and prints their CUDA-event times (the small case the
kernel profiles are captured on).
"""

from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-pt-steps/s at rel-L2<=1e-6 vs FP64; served p50/p99 latency vs plain"
UNIT = "grid-pt-steps/s"
N_GRID, L_BOX, T_END = 1024, 2.5, 2000.0
DU, DV, F, K = 2e-5, 1e-5, 0.035, 0.065
RTOL, ATOL, DT0, SEED = 1e-5, 1e-7, 1.0, 20261203
MAX_STEPS = 20000
SAVE_EVERY = 100  # t/dt history cadence; max_saves = MAX_STEPS // SAVE_EVERY + 1
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_GRID)
    ap.add_argument("--t-end", type=float, default=T_END)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp32"])
    ap.add_argument("--kernels-only", action="store_true")
    ap.add_argument("--graph", action="store_true", help="--kernels-only: time each kernel inside a CUDA graph")
    ap.add_argument("--workload", default="imex", choices=["imex", "etdrk4", "serve", "fft3d", "explicit", "nk", "stencil",
                                                          "gs256", "tubular"])
    ap.add_argument("--fp32", action="store_true", help="fft3d: FP32 instead of FP64")
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--no-configs", action="store_true", help="skip the configs 1, 3, 4, 5 legs of the default line")
    ap.add_argument("--etd-steps", type=int, default=100)
    ap.add_argument("--etd-method", default="etdrk4", choices=["etdrk4", "etd1", "etd2"])
    ap.add_argument("--reps", type=int, default=30)
    ap.add_argument("--adaptive", action="store_true", help="explicit: adaptive RK4 (step doubling, PI controller)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region (median SM clock, throttle reasons)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9 and parts[1].isdigit():
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]),
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ our arm
def make_problem(dtype, dev, n):
    import moljax_gb300 as M
    from moljax_gb300.workloads import gray_scott_initial_condition
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, DU, DV, F, K, dtype, dev)
    y0 = gray_scott_initial_condition(grid, SEED, dtype, dev)
    return M, grid, model, cache, diff, y0


def solve(M, model, cache, diff, y0, t_end, precision=None):
    pid = M.PIDParams(atol=ATOL, rtol=RTOL)
    return M.adaptive_integrate_imex(model, y0, 0.0, t_end, DT0, cache, diff, pid_params=pid,
                                     max_steps=MAX_STEPS, save_every=SAVE_EVERY,
                                     save_y_history=False, precision=precision)


def kernel_bytes(n, elem):
    """Algorithmic bytes of the seven passes of one attempt (2 fields, n x n)."""
    real = n * n * elem                  # one real field
    spec = n * (n // 2 + 1) * 2 * elem   # one half spectrum
    f = 2
    return {
        "K1 row r2c": f * (real + spec),
        "K2 col dual": f * (spec + 2 * spec),
        "K3 row c2r-react-r2c x2": 2 * f * (2 * spec),
        "K4 col x2": 2 * f * (2 * spec),
        "K5 row store|react": f * (spec + real) + f * (2 * spec),
        "K6 col": f * 2 * spec,
        "K7 row store+err": f * (spec + 2 * real),
    }


def kernel_bytes_mixed(n):
    """Algorithmic bytes of the six passes of one mixed-precision attempt (2 fields).

    Per field and half-spectrum element: float-float state/scratch 16 B, FP32 row spectra 8 B.
    """
    nc = n * (n // 2 + 1)
    f = 2
    return {"C1 col split": f * nc * 64, "R1 row delta x2": f * nc * 32,
            "C2 col combine": f * nc * 88, "R2 row delta": f * nc * 16,
            "C3 col end+err": f * nc * 72, "R3 row err": f * nc * 16}


def time_kernels_mixed(M, model, cache, diff, y0, dev, reps=30, graph=False):
    """CUDA-event time of each mixed-precision attempt kernel on the launching stream.  With
    graph=True each kernel is captured reps times back to back into a CUDA graph and the
    graph replayed (the kernel's cost inside the attempt loop, without the host's launch
    rate), and 'attempt' is the six kernels in order, captured 20 times."""
    import torch
    from moljax_gb300 import _native as N
    from moljax_gb300.core import stencil
    from moljax_gb300.core.fft_solvers import workspace, get_plan
    from moljax_gb300.core.stepping import _problem
    grid = model.grid
    interior = stencil.unpad(stencil.stack(y0, model.field_names), grid)
    p32 = get_plan(grid.ny, grid.nx, grid.dy, grid.dx, "fd", torch.float32, dev)
    p64 = get_plan(grid.ny, grid.nx, grid.dy, grid.dx, "fd", torch.float64, dev)
    prob = _problem(model, diff, M.CFLParams())
    pid = N.PIDParamsC(0.9, 0.7, 0.4, 1e-12, 1.0, 5.0, 0.2, ATOL, RTOL)
    lib = N.lib()
    ws = workspace(lib.mjx_imex2d_mixed_ws_bytes(grid.ny, grid.nx, 2), dev, "imex_mixed")
    stream = N.stream_ptr(dev)
    call = lambda w: N.check("mjx_imex_mixed_attempt_kernel2d", lib.mjx_imex_mixed_attempt_kernel2d(  # noqa
        N.ptr(p32.buf), N.ptr(p64.buf), C.byref(p32.cgrid), C.byref(prob), C.byref(pid), w, 0.9,
        N.ptr(interior), N.ptr(ws), ws.numel(), stream))
    call(0)
    names = list(kernel_bytes_mixed(grid.nx).keys())
    out = {}
    s = torch.cuda.current_stream(dev)
    if graph:
        for w in range(1, 7):
            call(w)
        torch.cuda.synchronize(dev)

        def graph_time(seq, n):
            g = torch.cuda.CUDAGraph()
            cs = torch.cuda.Stream(dev)
            cs.wait_stream(s)
            with torch.cuda.stream(cs):
                with torch.cuda.graph(g, stream=cs):
                    for _ in range(n):
                        for w in seq:
                            N.check("mjx_imex_mixed_attempt_kernel2d", lib.mjx_imex_mixed_attempt_kernel2d(
                                N.ptr(p32.buf), N.ptr(p64.buf), C.byref(p32.cgrid), C.byref(prob), C.byref(pid),
                                w, 0.9, N.ptr(interior), N.ptr(ws), ws.numel(), cs.cuda_stream))
            g.replay()
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(5):
                g.replay()
            e1.record(s)
            e1.synchronize()
            return e0.elapsed_time(e1) / 5 / n * 1e-3
        for w in range(1, 7):
            out[names[w - 1]] = graph_time([w], reps)
        out["attempt"] = graph_time([1, 2, 3, 4, 5, 6], 20)
        return out
    for w in range(1, 7):
        for _ in range(min(3, reps)):
            call(w)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            call(w)
        e1.record(s)
        e1.synchronize()
        out[names[w - 1]] = e0.elapsed_time(e1) / reps * 1e-3
    return out


def time_kernels(M, model, cache, diff, y0, dev, reps=30):
    """CUDA-event time of each FP32 attempt kernel on the launching stream."""
    import torch
    from moljax_gb300 import _native as N
    from moljax_gb300.core import stencil
    from moljax_gb300.core.fft_solvers import workspace, _plan_of
    from moljax_gb300.core.stepping import _problem
    grid = model.grid
    interior = stencil.unpad(stencil.stack(y0, model.field_names), grid)
    plan = _plan_of(cache, grid.ny, grid.nx, interior.dtype)
    prob = _problem(model, diff, M.CFLParams())
    pid = N.PIDParamsC(0.9, 0.7, 0.4, 1e-12, 1.0, 5.0, 0.2, ATOL, RTOL)
    lib = N.lib()
    ws = workspace(lib.mjx_imex2d_ws_bytes(grid.ny, grid.nx, 2, plan.code), dev, "imex")
    stream = N.stream_ptr(dev)
    call = lambda w: N.check("mjx_imex_attempt_kernel2d", lib.mjx_imex_attempt_kernel2d(  # noqa
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, C.byref(prob), C.byref(pid), w, 0.9,
        N.ptr(interior), N.ptr(ws), ws.numel(), stream))
    call(0)
    names = list(kernel_bytes(grid.nx, interior.element_size()).keys())
    out = {}
    s = torch.cuda.current_stream(dev)
    for w in range(1, 8):
        for _ in range(min(3, reps)):
            call(w)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            call(w)
        e1.record(s)
        e1.synchronize()
        out[names[w - 1]] = e0.elapsed_time(e1) / reps * 1e-3
    return out


def reduce_over_ranks(t_dev, units, device):
    """Replica aggregation: the slowest rank's time and every rank's units (the path does
    not shard, so there is no data-path collective; this is the only one)."""
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t_dev, float(units)], dtype=torch.float64, device=device)
    tmax = tt[:1].clone()
    tsum = tt[1:].clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    return float(tmax.item()), int(tsum.item())


def flush_l2(buf):
    buf.add_(1.0)


def run_ours(args, rank, world, local):
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    M, grid, model, cache, diff, y0 = make_problem(torch.float32, dev, args.n)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev)
    P = args.precision
    for _ in range(args.warmup):
        r = solve(M, model, cache, diff, y0, args.t_end, P)
    torch.cuda.synchronize(dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    clocks = Clocks(local)
    s = torch.cuda.current_stream(dev)
    times, units, attempts = [], 0, 0
    barrier()
    torch.cuda.synchronize(dev)
    clocks.start()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush_l2(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        r = solve(M, model, cache, diff, y0, args.t_end, P)
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
        units += grid.nx * grid.ny * r.n_accepted
        attempts += r.n_accepted + r.n_rejected
    torch.cuda.synchronize(dev)
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    t_dev = sum(times)
    if world > 1:
        t_dev, units = reduce_over_ranks(t_dev, units, dev)
    status = r.status
    n_acc, n_rej = r.n_accepted, r.n_rejected
    y32 = {k: v.detach().clone() for k, v in r.y_final.items()}

    # end to end through the public API with pinned host buffers (copies timed)
    host_in = {k: v.detach().cpu().pin_memory() for k, v in y0.items()}
    host_out = {k: torch.empty_like(v) .pin_memory() for k, v in host_in.items()}
    bi = sum(v.numel() * v.element_size() for v in host_in.values())
    bo = bi
    etimes, eunits = [], 0
    for _ in range(args.steps):
        flush_l2(flush)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        yd = {k: v.to(dev, non_blocking=True) for k, v in host_in.items()}
        rr = solve(M, model, cache, diff, yd, args.t_end, P)
        for k in host_out:
            host_out[k].copy_(rr.y_final[k], non_blocking=True)
        e1.record(s)
        e1.synchronize()
        etimes.append(e0.elapsed_time(e1) * 1e-3)
        eunits += grid.nx * grid.ny * rr.n_accepted

    out = {}
    if rank == 0:
        # error of the FP32 result against the FP64 GPU path (pinned to the FP64 oracle in tests)
        err = None
        fp64 = None
        other = None
        if not args.no_fp64:
            M2, g2, m64, c64, d64, y64 = make_problem(torch.float64, dev, args.n)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            r64 = solve(M2, m64, c64, d64, y64, args.t_end)
            e1.record(s)
            e1.synchronize()
            t64 = e0.elapsed_time(e1) * 1e-3
            num = sum(float(torch.linalg.norm(y32[k].double() - r64.y_final[k])) ** 2 for k in y32)
            den = sum(float(torch.linalg.norm(r64.y_final[k])) ** 2 for k in y32)
            err = (num / den) ** 0.5
            fp64 = {"value": g2.nx * g2.ny * r64.n_accepted / t64, "ms_per_solve": t64 * 1e3,
                    "n_accepted": r64.n_accepted, "n_rejected": r64.n_rejected}
            # the other single-precision form, for comparison
            Q = "fp32" if P == "mixed" else "mixed"
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            rq = solve(M, model, cache, diff, y0, args.t_end, Q)
            e1.record(s)
            e1.synchronize()
            tq = e0.elapsed_time(e1) * 1e-3
            nq = sum(float(torch.linalg.norm(rq.y_final[k].double() - r64.y_final[k])) ** 2 for k in y32)
            other = {"precision": Q, "value": g2.nx * g2.ny * rq.n_accepted / tq,
                     "ms_per_solve": tq * 1e3, "rel_l2_vs_fp64": (nq / den) ** 0.5,
                     "n_accepted": rq.n_accepted, "n_rejected": rq.n_rejected}
        # live per-kernel timing for the roofline of the dominant kernel
        if P == "mixed":
            ktimes = time_kernels_mixed(M, model, cache, diff, y0, dev)
            kb = kernel_bytes_mixed(grid.nx)
        else:
            ktimes = time_kernels(M, model, cache, diff, y0, dev)
            kb = kernel_bytes(grid.nx, 4)
        dom = max(ktimes, key=lambda k: ktimes[k])
        peak, peak_kind = peaks()
        achieved = kb[dom] / ktimes[dom] / 1e9
        traffic = None
        tp = os.path.join(ROOT, "profiles", "traffic_imex_gs1024.json")
        if os.path.exists(tp):
            with open(tp) as f:
                traffic = json.load(f).get(dom)
        out = {
            "metric": METRIC, "value": units / t_dev, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_dev / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if P == "fp32" else "f32 transforms + float-float (f32 pair) spectral state", "data": "synthetic",
            "config": {"workload": f"gray-scott IMEX-Strang adaptive {grid.ny}x{grid.nx} FP32, "
                                   f"t_span=(0,{args.t_end:g}), rtol={RTOL}, atol={ATOL}, "
                                   "Du=2e-5 Dv=1e-5 F=0.035 k=0.065 L=2.5",
                       "step": "one full adaptive solve", "parallelism": "replicas" if world > 1 else "1 GPU",
                       "l2": "flushed between timed solves (256 MB write); the 1024^2 working set "
                             "(~50 MB) stays L2-resident within a solve",
                       "n_accepted": n_acc, "n_rejected": n_rej, "status": status},
            "precision": P,
            "rel_l2_vs_fp64": err,
            "fp64_plain": fp64,
            "other_precision": other,
            "e2e": {"value": eunits / sum(etimes), "unit": UNIT, "h2d_bytes_per_step": bi,
                    "d2h_bytes_per_step": bo},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak,
                         "peak_kind": f"of {peak_kind}", "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "alg_bytes": kb[dom],
                         "kernel_us": {k: v * 1e6 for k, v in ktimes.items()}},
            # the graph body holds 4 attempts (mixed: 6 kernels + controller each; FP32: 7 + 1),
            # so a solve launches its attempts rounded up to a multiple of 4 (the surplus
            # kernels return at entry) plus its conversion kernels (mixed 9, FP32 3)
            "gpu_launches": args.steps * (-(-(attempts // args.steps) // 4) * 4 * (7 if P == "mixed" else 8)
                                          + (9 if P == "mixed" else 3)),
            "clocks": clk,
            "wall_s": wall,
        }
        if not args.no_configs:
            # the other benchmark configurations, each measured on its own terms
            out["configs"] = {"fft_cn_128": fftcn_leg(dev), "etdrk4_4096": etdrk4_leg(dev),
                              "nk_bdf2_512": nk_leg(dev), "served_mix": served_mix(dev, args.requests),
                              "stencil_gs_4096": stencil_gs_leg(dev), "tubular_rk4_sweep": tubular_leg(dev),
                              "gray_scott_256_methods": gs_methods_leg(dev)}
        if not args.no_cpu_baseline and world == 1:
            out["cpu_baseline"] = cpu_baseline(args)
    return out


def etd_kernel_bytes(n):
    """Algorithmic bytes of the 8 ETDRK4 passes of one step (2 fields, FP32): per field and
    half-spectrum element, complex 8 B / coefficient 4 B accesses (C1 5+2, R1 2, C2 4+2, R2 2,
    C3 6+2, R3 2, C4 6+4, R4 2)."""
    nc = n * (n // 2 + 1)
    per = {"C1": 5 * 8 + 2 * 4, "R1": 16, "C2": 4 * 8 + 2 * 4, "R2": 16, "C3": 6 * 8 + 2 * 4,
           "R3": 16, "C4": 6 * 8 + 4 * 4, "R4": 16}
    return {k: 2 * nc * v for k, v in per.items()}


def etd12_step_bytes(n, method):
    """Algorithmic bytes of one ETD1 / ETD2 step (2 fields, FP32): per field and half-spectrum
    element, column pass ETD1 4 complex + 2 coefficient accesses, ETD2 6 + 3; row pass 2."""
    nc = n * (n // 2 + 1)
    col = 4 * 8 + 2 * 4 if method == "etd1" else 6 * 8 + 3 * 4
    return 2 * nc * (col + 16)


def run_etd12(args, local):
    """Fixed-step coupled ETD1 / ETD2 Gray-Scott (FP32 state, FP64 phi coefficients) at n^2
    through etd_integrate: grid-pt-steps/s and the step-level achieved bandwidth."""
    import torch
    import moljax_gb300 as M
    from moljax_gb300.workloads import gray_scott_initial_condition
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n, S = args.n, args.etd_steps
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    y0 = gray_scott_initial_condition(grid, SEED, torch.float32, dev)
    g = grid.n_ghost
    st = {k: y0[k][g:g + n, g:g + n].contiguous() for k in ("u", "v")}
    ops = {"u": M.DiffusionOperator(grid, DU, torch.float32), "v": M.DiffusionOperator(grid, DV, torch.float32)}
    nl = M.NativeNonlinear.gray_scott(F, K)
    M.etd_integrate(st, (0.0, 3.0), 1.0, ops, nl, method=args.etd_method, save_every=3)
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    M.etd_integrate(st, (0.0, float(S)), 1.0, ops, nl, method=args.etd_method, save_every=S)
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    b = etd12_step_bytes(n, args.etd_method)
    peak, peak_kind = peaks()
    gbs = b * S / t / 1e9
    return {"workload": f"gray-scott {args.etd_method.upper()} {n}x{n} FP32, dt=1", "n": n, "steps": S,
            "value": n * n * S / t, "unit": UNIT, "ms_per_step": t / S * 1e3, "step_alg_bytes": b,
            "achieved_gbs": gbs, "frac_of_" + peak_kind.replace(" ", "_"): gbs / peak}


def run_etdrk4(args, local):
    """Fixed-step coupled ETDRK4 Gray-Scott (FP32 state, FP64 contour coefficients) at n^2:
    grid-pt-steps/s over --etd-steps steps, and the live per-pass roofline."""
    if args.etd_method != "etdrk4":
        return run_etd12(args, local)
    import torch
    import moljax_gb300 as M
    from moljax_gb300 import _native as N
    from moljax_gb300.core.fft_solvers import get_plan, workspace
    from moljax_gb300.workloads import gray_scott_initial_condition
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = args.n
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    model = M.create_gray_scott_model(grid, DU, DV, F, K, dtype=torch.float32)
    y0 = gray_scott_initial_condition(grid, SEED, torch.float32, dev)
    out = {"workload": f"gray-scott ETDRK4 {n}x{n} FP32, dt=1", "n": n, "steps": args.etd_steps}
    if not args.kernels_only:
        M.etdrk4_gray_scott(model, y0, 1.0, 3)
        torch.cuda.synchronize(dev)
        s = torch.cuda.current_stream(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        M.etdrk4_gray_scott(model, y0, 1.0, args.etd_steps)
        e1.record(s)
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        out["value"] = n * n * args.etd_steps / t
        out["unit"] = UNIT
        out["ms_per_step"] = t / args.etd_steps * 1e3
    # per-pass timing through the single-kernel entry (workspace left by the run above)
    plan = get_plan(n, n, grid.dy, grid.dx, "fd", torch.float32, dev)
    lib = N.lib()
    ws = workspace(lib.mjx_etdrk4_ws_bytes(n, n, plan.code), plan.device, "etd")
    if args.kernels_only:
        M.etdrk4_gray_scott(model, y0, 1.0, 1)
    names = list(etd_kernel_bytes(n).keys())
    order = [1, 2, 3, 4, 5, 6, 7, 8]
    reps = args.reps
    kt = {}
    s = torch.cuda.current_stream(dev)
    for w in order:
        call = lambda: N.check("mjx_etdrk4_kernel2d", lib.mjx_etdrk4_kernel2d(  # noqa: E731
            N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, F, K, w, N.ptr(ws), ws.numel(),
            N.stream_ptr(dev)))
        for _ in range(min(3, reps)):
            call()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            call()
        e1.record(s)
        e1.synchronize()
        kt[names[w - 1]] = e0.elapsed_time(e1) / reps * 1e-3
    kb = etd_kernel_bytes(n)
    peak, peak_kind = peaks()
    out["kernel_us"] = {k: v * 1e6 for k, v in kt.items()}
    out["kernel_gbs"] = {k: kb[k] / kt[k] / 1e9 for k in kt}
    out["step_alg_bytes"] = sum(kb.values())
    if "value" in out:
        out["achieved_gbs"] = sum(kb.values()) / (out["ms_per_step"] * 1e-3) / 1e9
        out["frac_of_" + peak_kind.replace(" ", "_")] = out["achieved_gbs"] / peak
    return out


def run_fft3d(args, local):
    """3D FFT-CN diffusion (benchmarks/sisc/bench_3d_feasibility.py: D = 0.1, T = 0.01 in 10
    steps, spectral symbol) at n^3: the published case (10 steps) timed as the reference
    times it, plus --etd-steps steps for throughput and the HBM roofline of a step (five
    passes, each reading and writing the box: 80 B per point FP64, 40 B FP32)."""
    import numpy as np
    import torch
    import moljax_gb300 as M
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = args.n
    dt_ = torch.float32 if args.fp32 else torch.float64
    x = torch.arange(n, dtype=torch.float64, device=dev) / n
    s1 = torch.sin(2 * math.pi * x)
    u0 = (s1[:, None, None] * s1[None, :, None] * s1[None, None, :]).to(dt_).contiguous()
    D, T, n10 = 0.1, 0.01, 10
    dt = T / n10
    for _ in range(3):
        M.fft_cn_step_3d(u0, D, 1.0 / n, dt, n10)
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    times = []
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        u = M.fft_cn_step_3d(u0, D, 1.0 / n, dt, n10)
        e1.record(s)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    exact = u0.double() * math.exp(-12 * math.pi ** 2 * D * T)
    err = float((u.double() - exact).abs().max())
    S = args.etd_steps
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    M.fft_cn_step_3d(u0, D, 1.0 / n, dt, S)
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    per_pt = 80 if dt_ == torch.float64 else 40
    b = per_pt * n ** 3
    peak, peak_kind = peaks()
    gbs = b * S / t / 1e9
    return {"workload": f"3D FFT-CN diffusion {n}^3 {'FP32' if args.fp32 else 'FP64'}, spectral symbol",
            "n": n, "published_case_ms": float(np.median(times)), "published_case_max_error": err,
            "steps": S, "value": n ** 3 * S / t, "unit": UNIT, "ms_per_step": t / S * 1e3,
            "step_alg_bytes": b, "achieved_gbs": gbs, "frac_of_" + peak_kind.replace(" ", "_"): gbs / peak}


def run_explicit(args, local):
    """Fixed-step RK4 of the two-species advection-diffusion model (examples/advdiff_multispecies.py
    shape: D = 1e-4, v = (0.5, -0.3), upwind, periodic) at n^2 in FP32: grid-pt-steps/s over
    --etd-steps steps and the HBM roofline of a step.  Per field and point an RK4 step makes
    16 buffer accesses in its four fused stage kernels (3 + 5 + 5 + 3: stage input, step
    start, running sum; outputs), 64 B in FP32."""
    import numpy as np
    import torch
    import moljax_gb300 as M
    from moljax_gb300.core.stepping import _explicit_steps
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n, S = args.n, args.etd_steps
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_advection_diffusion_model(grid, field_names=("c1", "c2"), D=1e-4, vx=0.5, vy=-0.3,
                                               dtype=torch.float32)
    rng = np.random.default_rng(SEED)
    y0 = {k: torch.tensor(rng.uniform(0, 1, (n + 2, n + 2)), dtype=torch.float32, device=dev) for k in ("c1", "c2")}
    dt = 0.2 * min(grid.dx / 0.8, grid.dx ** 2 / (4 * 1e-4))
    if args.adaptive:
        return run_explicit_adaptive(args, model, y0, dt, n, S, dev)
    _explicit_steps(model, y0, 0.0, dt, 2, 3)
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    _explicit_steps(model, y0, 0.0, dt, 2, S)
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    b = 2 * n * n * 64
    bf = 2 * n * n * 8
    peak, peak_kind = peaks()
    gbs = b * S / t / 1e9
    out = {"workload": f"advection-diffusion RK4 2 fields {n}x{n} FP32, upwind, periodic", "n": n, "steps": S,
           "value": n * n * S / t, "unit": UNIT, "ms_per_step": t / S * 1e3,
           "unfused_step_bytes": b, "unfused_equivalent_gbs": gbs,
           "fused_step_bytes": bf, "fused_dram_gbs": bf * S / t / 1e9,
           "fused_dram_frac_of_" + peak_kind.replace(" ", "_"): bf * S / t / 1e9 / peak,
           "bound": "instruction issue in the fused step (one kernel per RK4 step, stages in shared memory)",
           "gpu_launches": S}
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = explicit_cpu_baseline()
    return out


def run_explicit_adaptive(args, model, y0, dt, n, S, dev):
    """adaptive_integrate with RK4 (step doubling: a full step and two half steps per
    attempt, 12 stencil-stage launches, the error fused into the last; PI controller and
    CFL limit on the device in a conditional graph) for S attempts from t = 0, no state
    history.  Reports attempts/s, accepted pt-steps/s and the stage kernels' HBM rate
    (12 stages x 16/4 accesses: 48 accesses = 192 B per point and field per attempt in
    FP32)."""
    import torch
    import moljax_gb300 as M
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    kw = dict(method=M.IntegratorType.RK4, max_steps=10 * S + 10, pid_params=pid, save_every=1,
              save_y_history=False)
    M.adaptive_integrate(model, y0, 0.0, 1e9, dt, max_attempts=8, **kw)  # tunes and captures
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    r = M.adaptive_integrate(model, y0, 0.0, 1e9, dt, max_attempts=S, **kw)
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    att = r.n_accepted + r.n_rejected
    b = 2 * n * n * 192
    peak, peak_kind = peaks()
    return {"workload": f"advection-diffusion adaptive RK4 (step doubling) 2 fields {n}x{n} FP32, upwind, periodic, "
                        f"rtol=1e-5, atol=1e-7", "n": n, "attempts": att, "n_accepted": r.n_accepted,
            "n_rejected": r.n_rejected, "t_reached": float(r.t_final), "ms_per_attempt": t / max(att, 1) * 1e3,
            "value": n * n * r.n_accepted / t, "unit": UNIT, "attempt_alg_bytes": b,
            "achieved_gbs": b * att / t / 1e9, "frac_of_" + peak_kind: b * att / t / 1e9 / peak,
            "stencil_rows": M.autotune.stencil_rows(n, n, 2, torch.float32)}


def explicit_cpu_baseline(n=1024, steps=48):
    """The oracle's RK4 of the same model (NumPy FP64, one core) on a bounded sample."""
    import numpy as np
    from oracle import explicit as OX
    from oracle import mol
    og = mol.Grid2D(n, n, 0, 1, 0, 1)
    om = OX.ExplicitModel(og, {"c1": mol.PERIODIC, "c2": mol.PERIODIC}, {"c1": 1e-4, "c2": 1e-4},
                          advection="upwind", vx=0.5, vy=-0.3, params={"D": 1e-4, "vx": 0.5, "vy": -0.3})
    rng = np.random.default_rng(SEED)
    y = {k: mol.pad(rng.uniform(0, 1, (n, n)), og) for k in ("c1", "c2")}
    dt = 0.2 * min(og.dx / 0.8, og.dx ** 2 / (4 * 1e-4))
    t0 = time.perf_counter()
    for _ in range(steps):
        y = OX.rk4_step(om, y, dt)
    d = time.perf_counter() - t0
    return {"value": n * n * steps / d, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} RK4 steps of the same model at {n}^2 in {d:.1f} s (NumPy FP64 restatement)"}


def run_stencil(args, local):
    """The stencil stage kernel alone (rk_stage_tma_kernel / rk_stage_vec_kernel /
    rk_stage_kernel): one RK4 middle stage of the two-field advection-diffusion model of
    the explicit workload at n^2, timed by the autotuner for each tile height and the
    TMA-staged form (64; FP32) (CUDA events, 20 launches each after a warm-up launch).  Algorithmic bytes per point and field: stage input, step start and
    running sum read, two outputs written = 5 accesses (20 B in FP32, 40 B in FP64); the
    5-point neighbours come from cache."""
    import torch
    import moljax_gb300 as M
    from moljax_gb300.core import autotune as AT
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = args.n
    dtype = torch.float32 if args.fp32 else torch.float64
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_advection_diffusion_model(grid, ("c1", "c2"), D=1e-4, vx=0.5, vy=-0.3, dtype=dtype)
    res = AT.autotune_stencil(model, dtype, reps=20)
    esz = 4 if dtype == torch.float32 else 8
    b = 2 * n * n * 5 * esz
    peak, peak_kind = peaks()
    t = min(res.times_ms) * 1e-3
    return {"workload": f"stencil stage (RK4 middle stage) advection-diffusion 2 fields {n}x{n} "
                        f"{'FP32' if dtype == torch.float32 else 'FP64'}",
            "n": n, "kernel": ("rk_stage_tma_kernel" if res.choice[0] == 64 else
                               "rk_stage_vec_kernel" if n % (16 // esz) == 0 else "rk_stage_kernel"),
            "tile_heights": [c[0] for c in res.candidates], "ms_per_launch": res.times_ms,
            "best_rows": res.choice[0], "alg_bytes": b,
            "roofline": {"bound": "hbm", "achieved": b / t / 1e9, "peak": peak, "peak_kind": peak_kind,
                         "unit": "GB/s", "frac": b / t / 1e9 / peak}}


def run_nk(args, local):
    """Fixed-step BDF2 (BE first step) of u_t = div((1 + u^2) grad u) - u^3 on the unit square
    with Dirichlet walls at n^2 cell centres, u0 a seeded sum of 8 Gaussians (A ~ U[0,1],
    w ~ U[0.02,0.1]), dt = 100 dx^2, GMRES(30), Newton rtol 1e-8: FP64 state and residual,
    FP32 Krylov, through the native Newton-Krylov driver.  Reports ms per step and the
    Newton / GMRES iterations per step."""
    import numpy as np
    import torch
    import moljax_gb300 as M
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n, S = args.n, args.etd_steps
    dx = 1.0 / n
    rng = np.random.default_rng(SEED)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    u0 = np.zeros((n, n))
    for _ in range(8):
        A, w = rng.uniform(0.0, 1.0), rng.uniform(0.02, 0.1)
        cx, cy = rng.uniform(0.0, 1.0, 2)
        u0 += A * np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * w * w))
    u0 = torch.tensor(u0, device=dev)
    dt = 100 * dx * dx
    nkp = M.NKParams(gmres_restart=30)
    M.integrate_implicit_vardiff(u0, dx, dt, 3, method="bdf2", nk_params=nkp, be_guess="previous")
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    u, st = M.integrate_implicit_vardiff(u0, dx, dt, S, method="bdf2", nk_params=nkp, be_guess="previous")
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    out = {"workload": f"variable-diffusion BDF2 Newton-Krylov {n}x{n} FP64/FP32-Krylov (Dirichlet), dt=100dx^2",
           "n": n, "steps": S, "value": n * n * S / t, "unit": UNIT, "ms_per_step": t / S * 1e3,
           "newton_per_step": float(st[:, 0].double().mean()), "gmres_per_step": float(st[:, 1].double().mean()),
           "all_converged": bool((st[:, 2] != 0).all())}
    if not args.no_cpu_baseline:
        from oracle import nk as ONK
        m, steps = min(n, 256), 16
        dxm = 1.0 / m
        u0c = ONK.gaussians_ic(m, seed=SEED % 1000)
        t0 = time.perf_counter()
        ONK.bdf2_integrate(u0c, dxm, dxm, 100 * dxm * dxm, steps, restart=30, be_guess="previous")
        d = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": m * m * steps / d, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": f"{steps} BDF2 steps at {m}^2 in {d:.1f} s (NumPy/SciPy FP64 Newton-GMRES(30) "
                                         f"restatement with the DST preconditioner)"}
    return out


def fftcn_leg(dev):
    """Config 1: FFT-CN 128^2 on [0,1)^2 (node grid), FP64, D = 0.1, dt = 0.01, 100 steps one
    by one through fft_solvers.fft_cn_step, pseudo-spectral symbol; absolute pt-steps/s (the
    128^2 field sits on chip, so the pass is latency-bound and no roofline applies) and the
    error against the analytic decay exp(-8 pi^2 D t) (CN truncation 4.1e-3 relative)."""
    import torch
    import moljax_gb300 as M
    n, D, dt, S = 128, 0.1, 0.01, 100
    x = torch.arange(n, dtype=torch.float64, device=dev) / n
    u0 = (torch.sin(2 * math.pi * x)[:, None] * torch.sin(2 * math.pi * x)[None, :]).contiguous()
    for _ in range(3):
        M.fft_cn_step(u0, D, 1.0 / n, dt, S)
    torch.cuda.synchronize(dev)
    s = torch.cuda.current_stream(dev)
    ts = []
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        u = M.fft_cn_step(u0, D, 1.0 / n, dt, S)
        e1.record(s)
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = min(ts)
    exact = u0 * math.exp(-8 * math.pi ** 2 * D * dt * S)
    rel = float(torch.linalg.norm(u - exact) / torch.linalg.norm(exact))
    return {"workload": "FFT-CN 2D periodic diffusion 128x128 FP64, D=0.1, dt=0.01, 100 steps (fft_cn_step)",
            "value": n * n * S / t, "unit": UNIT, "ms_per_solve": t * 1e3, "us_per_step": t / S * 1e6,
            "rel_l2_vs_analytic_decay": rel, "gpu_launches_per_solve": 3 * S,
            "roofline": "latency-bound (128^2 FP64 field, 128 KB, on chip): absolute throughput only"}


def nk_leg(dev, n=512, steps=20):
    """Config 4: NK-BDF2 at 512^2 (run_nk) plus the achieved bandwidth by the byte
    convention per GMRES iteration j of a cycle, (11 + 2 j) b per point (JVP 3b, DST
    preconditioner 6b, Arnoldi (2j + 2) b, b = 4), and 32 B per point per Newton residual."""
    import types
    out = run_nk(types.SimpleNamespace(n=n, etd_steps=steps, no_cpu_baseline=True), dev.index or 0)
    g_per_newton = out["gmres_per_step"] / max(out["newton_per_step"], 1e-9)
    jbar = max(g_per_newton - 1.0, 0.0) / 2.0
    bytes_step = n * n * (out["gmres_per_step"] * (11 + 2 * jbar) * 4 + out["newton_per_step"] * 32)
    peak, peak_kind = peaks()
    gbs = bytes_step / (out["ms_per_step"] * 1e-3) / 1e9
    out["alg_bytes_per_step"] = bytes_step
    out["achieved_gbs"] = gbs
    out["frac_of_" + peak_kind] = gbs / peak
    out["bound"] = ("latency (L2-resident): six kernels per GMRES iteration (JVP, three DST passes, "
                    "dots, orthogonalisation) plus two FP64 residuals per Newton iteration")
    return out


def etdrk4_leg(dev, n=4096, steps=100, err_steps=10):
    """Config 3: coupled Gray-Scott ETDRK4 at 4096^2, FP32 state with FP64 contour
    coefficients, dt = 1 (run_etdrk4: throughput and per-pass roofline), plus the FP32
    against FP64 relative L2 error after err_steps steps from the same initial state."""
    import types
    import torch
    import moljax_gb300 as M
    from moljax_gb300.workloads import gray_scott_initial_condition
    out = run_etdrk4(types.SimpleNamespace(n=n, etd_steps=steps, kernels_only=False, reps=10,
                                           etd_method="etdrk4"), dev.index or 0)
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    y32 = gray_scott_initial_condition(grid, SEED, torch.float32, dev)
    y64 = {k: v.double() for k, v in y32.items()}
    r32 = M.etdrk4_gray_scott(M.create_gray_scott_model(grid, DU, DV, F, K, dtype=torch.float32), y32, 1.0, err_steps)
    r64 = M.etdrk4_gray_scott(M.create_gray_scott_model(grid, DU, DV, F, K, dtype=torch.float64), y64, 1.0, err_steps)
    num = sum(float(torch.linalg.norm(r32[k].double() - r64[k])) ** 2 for k in ("u", "v"))
    den = sum(float(torch.linalg.norm(r64[k])) ** 2 for k in ("u", "v"))
    out["fp32_rel_l2_vs_fp64"] = (num / den) ** 0.5
    out["error_steps"] = err_steps
    return out


def stencil_gs_leg(dev, n=4096):
    """The fused 5-point stencil + Gray-Scott reaction stage of the explicit steppers (an RK4
    middle stage: stage input, step start and running sum read, two outputs written =
    20 B per point and field in FP32) on a 4096^2 two-field grid, periodic, timed by the
    autotuner for every tile height and the TMA-staged form (20 launches each, CUDA
    events); the fastest candidate's rate against the measured HBM peak."""
    import torch
    import moljax_gb300 as M
    from moljax_gb300.core import autotune as AT
    grid = M.Grid2D(n, n, 0.0, L_BOX, 0.0, L_BOX)
    model = M.create_gray_scott_model(grid, DU, DV, F, K, dtype=torch.float32)
    with torch.cuda.device(dev):
        res = AT.autotune_stencil(model, torch.float32, reps=20, device=dev)
    b = 2 * n * n * 5 * 4
    t = min(res.times_ms) * 1e-3
    peak, peak_kind = peaks()
    best = res.choice[0]
    return {"workload": f"stencil + Gray-Scott reaction stage (RK4 middle stage) 2 fields {n}x{n} FP32, periodic",
            "kernel": "rk_stage_tma_kernel" if best == 64 else "rk_stage_vec_kernel", "best_rows": best,
            "candidates": [c[0] for c in res.candidates], "ms_per_launch": res.times_ms, "alg_bytes": b,
            "roofline": {"bound": "hbm", "achieved": b / t / 1e9, "peak": peak, "unit": "GB/s",
                         "peak_kind": peak_kind, "frac": b / t / 1e9 / peak}}


def gs_methods_leg(dev, steps_frac=1.0):
    """The reference's Gray-Scott method benchmark (benchmarks/benchmark_gray_scott.py,
    published in benchmarks/results/gray_scott.json): 256^2 on [0,1]^2, Du=2e-5, Dv=1e-5,
    F=0.035, k=0.065, pseudo-spectral Laplacian, its seed-42 initial condition, FP64, to
    t = 10 000: CN with the FFT-preconditioned Newton iteration (dt 0.5, 20 000 steps, tol
    1e-8, at most 10 iterations), the Strang exp-diffusion IMEX (dt 0.5, 20 000 steps), the
    benchmark's ETDRK4 (dt 1, 10 000 steps, 32-point contour coefficients) and the
    pseudo-spectral RK4 (dt 0.0974 = 0.9 of its stability limit, 102 669 steps).  Each method
    timed with CUDA events after a 10-step warm-up, against the published wall time of the
    reference on its own GPU (one run, the median of 10 there)."""
    import json
    import torch
    import moljax_gb300 as M
    from moljax_gb300.core import stencil
    from moljax_gb300.workloads import gray_scott_benchmark_ic
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "gray_scott_published.json")))
    cfg = g["config"]
    n = cfg["N"]
    pub = {m_["name"]: m_ for m_ in g["methods"]}
    Du, Dv, Fp, Kp = cfg["Du"], cfg["Dv"], cfg["F"], cfg["k"]
    dx = 1.0 / n
    u0, v0 = gray_scott_benchmark_ic(n, torch.float64, dev)
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_gray_scott_model(grid, Du, Dv, Fp, Kp, dtype=torch.float64)
    s = torch.cuda.current_stream(dev)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        r = fn()
        e1.record(s)
        e1.synchronize()
        return r, e0.elapsed_time(e1) * 1e-3

    def padded(u, v):
        return {k: t for k, t in zip(("u", "v"), stencil.pad_interior(torch.stack([u, v]), grid, model.bc_spec,
                                                                        ("u", "v")))}
    out = {"workload": "Gray-Scott 256^2 method benchmark (benchmark_gray_scott.py), FP64, pseudo-spectral, "
                       "t_final=10000", "published_hw": "reference's own GPU (RTX 5060), JAX FP64",
           "methods": {}}
    st = max(1, int(steps_frac * pub["CN (Newton-Krylov)"]["steps"]))
    M.gray_scott_cn_newton(u0, v0, Du, Dv, Fp, Kp, dt=0.5, n_steps=10, dx=dx)
    (u, v, its), t = timed(lambda: M.gray_scott_cn_newton(u0, v0, Du, Dv, Fp, Kp, dt=0.5, n_steps=st, dx=dx))
    its = its.cpu()
    out["methods"]["CN (Newton-Krylov)"] = {"steps": st, "time_s": t, "newton_per_step": float(its.double().mean()),
                                            "published_time_s": pub["CN (Newton-Krylov)"]["time_s"],
                                            "u_mean": float(u.mean())}
    st = max(1, int(steps_frac * pub["IMEX-Strang"]["steps"]))
    M.gray_scott_strang_exp(u0, v0, Du, Dv, Fp, Kp, 0.5, 10, dx)
    (u, v), t = timed(lambda: M.gray_scott_strang_exp(u0, v0, Du, Dv, Fp, Kp, 0.5, st, dx))
    out["methods"]["IMEX-Strang"] = {"steps": st, "time_s": t, "published_time_s": pub["IMEX-Strang"]["time_s"],
                                     "u_mean": float(u.mean())}
    st = max(1, int(steps_frac * pub["ETDRK4"]["steps"]))
    y0 = padded(u0, v0)
    M.etdrk4_gray_scott(model, y0, 1.0, 10, symbol="spectral", variant="benchmark")
    y, t = timed(lambda: M.etdrk4_gray_scott(model, y0, 1.0, st, symbol="spectral", variant="benchmark"))
    out["methods"]["ETDRK4"] = {"steps": st, "time_s": t, "published_time_s": pub["ETDRK4"]["time_s"],
                                "u_mean": float(y["u"][1:-1, 1:-1].mean())}
    rk = pub["RK4 (explicit)"]
    st = max(1, int(steps_frac * rk["steps"]))
    M.gray_scott_rk4_spectral(u0, v0, Du, Dv, Fp, Kp, rk["dt"], 10, dx)
    (u, v), t = timed(lambda: M.gray_scott_rk4_spectral(u0, v0, Du, Dv, Fp, Kp, rk["dt"], st, dx))
    out["methods"]["RK4 (explicit)"] = {"steps": st, "time_s": t, "published_time_s": rk["time_s"],
                                        "u_mean": float(u.mean())}
    for m_ in out["methods"].values():
        m_["value"] = n * n * m_["steps"] / m_["time_s"]
        m_["unit"] = UNIT
        m_["speedup_vs_published"] = m_["published_time_s"] / m_["time_s"] if steps_frac == 1.0 else None
    return out


def tubular_leg(dev):
    """The 27-case penalty-RK4 tubular-reactor sweep of benchmark_tubular_reactor.py (N = 128,
    t_final = 15, up to 967 740 RK4 steps per case, FP64) in one launch of the batched
    reactor kernel, timed with CUDA events after one warm-up sweep, against the sum of the
    reference's published per-case times (its own GPU, one case at a time); max relative
    deviation of the conversions from the published ones."""
    import json
    import torch
    from moljax_gb300.core import reactor as R
    g = json.load(open(os.path.join(ROOT, "tests", "golden", "tubular_published.json")))
    R.run_tubular_sweep(t_final=0.5, device=dev)
    s = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    res = R.run_tubular_sweep(N=g["N"], t_final=g["t_final"], dtype=torch.float64, device=dev)
    e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    pub = g["results"]
    dev_max = max(abs(res[k]["conversion"] - v["conversion"]) / max(abs(v["conversion"]), 1e-300)
                  for k, v in pub.items())
    steps = sum(v["n_steps"] for v in pub.values())
    return {"workload": "tubular reactor penalty-RK4 sweep, 27 cases (Danckwerts/Robin/Neumann x Pe 1,10,100 x "
                        "Da 0.1,1,10), N=128, t_final=15, FP64, one launch",
            "sweep_s": t, "published_sweep_s": sum(v["mean_time"] for v in pub.values()),
            "published_hw": "reference's own GPU (RTX 5060), one case at a time", "rk4_steps": steps,
            "value": g["N"] * steps / t, "unit": UNIT, "max_rel_dev_conversion_vs_published": dev_max,
            "gpu_launches": 1}


def served_mix(dev, n_requests, realtime=True, slots=64):
    """The served mix (config 5's Poisson arrivals at 2000/s, seed 5, its first n_requests
    requests): the continuous-batching server (FP32 + float-float Gray-Scott batch engine,
    batched reactor kernel) against the same requests solved one at a time in FP64 (the
    plain form of the same kernels), FIFO, no arrival waits.  Reports p50/p99 latency,
    solves/s and grid-point-steps/s of both, their ratio, and the largest rel-L2 of a
    served Gray-Scott result against its plain FP64 result."""
    import torch
    from moljax_gb300.serve import make_mix, Server, run_plain, summarize
    Server(dev, slots=8).run(make_mix(12, seed=99, gs_sizes=(64, 128)), realtime=False)  # warm kernels
    mix = make_mix(n_requests)
    srv = Server(dev, slots=slots)
    done = srv.run(mix, realtime=realtime)
    served = summarize(done, srv.makespan)
    served.update({"reactor_batches": srv.batches, "gs_epochs": srv.epochs, "slots": slots})
    plain = run_plain(mix, torch.float64, dev, realtime=False)
    pl = summarize(plain, max(c.end for c in plain))
    by_id = {c.rid: c for c in plain}
    err = 0.0
    for c in done:
        if c.kind == "gs":
            ref = by_id[c.rid].output
            err = max(err, float(torch.linalg.norm(c.output.double() - ref) / torch.linalg.norm(ref)))
    n_gs = sum(1 for r in mix if r.kind == "gs")
    return {"workload": f"served mix: first {n_requests} requests of the config-5 stream (Poisson 2000/s, seed 5; "
                        f"{n_gs} Gray-Scott 64^2..512^2 t_end=100, {n_requests - n_gs} reactor CN n=64..4096)",
            "served": served, "plain_fp64": pl,
            "speedup_pt_steps": served["pt_steps_per_s"] / pl["pt_steps_per_s"],
            "speedup_solves": served["solves_per_s"] / pl["solves_per_s"],
            "gs_max_rel_l2_vs_plain_fp64": err}


def run_serve(args, local):
    """--workload serve: the served mix with --requests requests (see served_mix)."""
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    return served_mix(dev, args.requests)


def run_kernels_only(args, local):
    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    M, grid, model, cache, diff, y0 = make_problem(torch.float32, dev, args.n)
    if args.precision == "mixed":
        kt = time_kernels_mixed(M, model, cache, diff, y0, dev, reps=args.reps, graph=args.graph)
    else:
        kt = time_kernels(M, model, cache, diff, y0, dev, reps=args.reps)
    return {"kernels_us": {k: v * 1e6 for k, v in kt.items()}, "precision": args.precision,
            "n": args.n, "reps": args.reps, "in_graph": bool(args.graph and args.precision == "mixed")}


# ------------------------------------------------------------------ CPU (oracle) arms
def cpu_sample(n, attempts, workers):
    """Adaptive IMEX-Strang on the CPU oracle for a bounded number of attempts."""
    from oracle import imex as OI, mol
    mol.set_fft_workers(workers)
    og = mol.Grid2D(n, n, 0, L_BOX, 0, L_BOX)
    om, lam, od = OI.gray_scott_periodic(og, DU, DV, F, K)
    y0 = mol.gray_scott_ic(og, SEED)
    t0 = time.perf_counter()
    r = OI.adaptive_integrate_imex(om, y0, 0.0, T_END, DT0, lam, od,
                                   pid=OI.PIDParams(atol=ATOL, rtol=RTOL), max_steps=MAX_STEPS,
                                   save_every=SAVE_EVERY, keep_history=False, max_attempts=attempts)
    dt = time.perf_counter() - t0
    return n * n * r.n_accepted / dt, r, dt


CPU_ATTEMPTS = 16  # attempts per CPU sample (about 2.5 s of the 1024^2 oracle on 16 Arm cores)


def cpu_baseline(args):
    """The oracle on the host cores: one untimed warm-up attempt, then one sample of
    CPU_ATTEMPTS attempts from t = 0 -- the same sampler and sample length as each step
    of the reference arm, so both report the same CPU figure."""
    workers = os.cpu_count() or 1
    cpu_sample(args.n, 1, workers)
    v, r, d = cpu_sample(args.n, CPU_ATTEMPTS, workers)
    return {"value": v, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{r.n_accepted + r.n_rejected} attempts of the same {args.n}^2 solve from t=0 "
                      f"({r.n_accepted} accepted, t reached {r.t_final:.3g}) in {d:.1f} s after a 1-attempt "
                      f"warm-up; NumPy/SciPy FP64 restatement, scipy.fft workers={workers}"}


def run_reference(args, rank, world):
    if rank != 0:
        return None
    workers = os.cpu_count() or 1
    for _ in range(max(1, args.warmup)):  # untimed: warms the FFT plans and caches
        cpu_sample(args.n, 1, workers)
    tot_units, tot_t = 0, 0.0
    for _ in range(args.steps):
        v, r, d = cpu_sample(args.n, CPU_ATTEMPTS, workers)
        tot_units += args.n * args.n * r.n_accepted
        tot_t += d
    value = tot_units / tot_t
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_t / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": f"gray-scott IMEX-Strang adaptive {args.n}x{args.n}, "
                                   f"t_span=(0,{T_END:g}), rtol={RTOL}, atol={ATOL}",
                       "step": f"{CPU_ATTEMPTS} attempts of the adaptive solve from t=0 (bounded CPU sample)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": workers, "kind": "port",
                             "sample": f"{CPU_ATTEMPTS} attempts per step from t=0, NumPy/SciPy FP64 restatement "
                                       "of the reference (JAX is not installed here or on the GPU host), "
                                       f"scipy.fft workers={workers}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        out = run_reference(args, rank, world)
    elif args.workload == "etdrk4":
        out = run_etdrk4(args, local)
    elif args.workload == "serve":
        out = run_serve(args, local)
    elif args.workload == "fft3d":
        out = run_fft3d(args, local)
    elif args.workload == "explicit":
        out = run_explicit(args, local)
    elif args.workload == "nk":
        out = run_nk(args, local)
    elif args.workload == "stencil":
        out = run_stencil(args, local)
    elif args.workload in ("gs256", "tubular"):
        import torch
        dev = torch.device("cuda", local)
        torch.cuda.set_device(dev)
        out = gs_methods_leg(dev) if args.workload == "gs256" else tubular_leg(dev)
    elif args.kernels_only:
        out = run_kernels_only(args, local)
    else:
        out = run_ours(args, rank, world, local)
    if rank == 0 and out:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
