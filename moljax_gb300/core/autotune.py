"""Autotuner of the native launch choices.

Two families of choices are timed on the device (CUDA events, native timing loops in
``csrc/dftn.cu`` and ``csrc/explicit.cu``) and the fastest is installed in the
library's process-wide registry, which the launchers read:

* the radix schedule of a mixed-radix DFT length n = 2^a 3^b 5^c (the order of the
  radix-2/3/4/5 Stockham passes, and powers of two as radix-4 or radix-2 passes) with
  the threads per sequence, used by every general-size periodic plan (2D and 3D);
* the tile height (rows per warp strip) of the explicit stencil stage kernel per grid
  size, field count and dtype, used by the adaptive explicit loop, Euler steps and
  ``MOLModel.rhs``.

The reference has no counterpart (under ``jax.jit`` XLA picks its own FFT and fusion
strategies: moljax/core/fft_solvers.py:33-80, moljax/core/stepping.py:126-163).

Plans of non-power-of-two sizes and the first adaptive explicit solve of a size tune
themselves once per process unless ``MJX_AUTOTUNE=0``.  ``save`` / ``load`` keep the
choices across processes (a JSON file), ``MJX_AUTOTUNE_CACHE`` names one to load on
first use.  Every candidate computes the same transform or stencil; schedules differ
only in rounding (the GPU tests check each against NumPy).
"""

from __future__ import annotations

import ctypes as C
import json
import os
from typing import Dict, List, NamedTuple, Optional, Sequence, Tuple

import torch

from moljax_gb300 import _native as N

_DFT_DONE: set = set()       # (n, dtype code) tuned or loaded in this process
_STENCIL_DONE: set = set()   # (ny, nx, nf, dtype code)
_RECORD: Dict[str, dict] = {}  # installed choices, for save()
_CACHE_LOADED = False


class TuneResult(NamedTuple):
    choice: tuple            # DFT: (schedule, tpsm); stencil: (rows,)
    candidates: List[tuple]  # same form as choice, in timing order
    times_ms: List[float]    # per launch, one per candidate
    best: int                # index of the winner


def enabled() -> bool:
    return os.environ.get("MJX_AUTOTUNE", "1") != "0"


def _maybe_load_cache():
    global _CACHE_LOADED
    if _CACHE_LOADED:
        return
    _CACHE_LOADED = True
    path = os.environ.get("MJX_AUTOTUNE_CACHE")
    if path and os.path.exists(path):
        load(path)


# ---- DFT schedules ---------------------------------------------------------------

def dft_schedule_candidates(n: int) -> List[Tuple[int, ...]]:
    """The candidate radix schedules of length n (host only; empty for powers of two and
    lengths with a prime factor above 5)."""
    buf = (C.c_int * (17 * 64))()
    k = N.lib().mjx_dft_schedule_candidates(int(n), buf, 64)
    return [tuple(buf[17 * i + 1: 17 * i + 1 + buf[17 * i]]) for i in range(k)]


def dft_schedule(n: int, dtype: torch.dtype = torch.float64) -> Tuple[Tuple[int, ...], int]:
    """(schedule, threads per sequence) in use for length n; ((), 0) when n has none."""
    nrad, tp = C.c_int(), C.c_int()
    rad = (C.c_int * 16)()
    N.check("mjx_dft_schedule_get", N.lib().mjx_dft_schedule_get(int(n), N.dtype_code(dtype), C.byref(nrad),
                                                                 rad, C.byref(tp)))
    return tuple(rad[: nrad.value]), tp.value


def set_dft_schedule(n: int, dtype: torch.dtype, schedule: Sequence[int], tpsm: int = 0) -> None:
    """Install a schedule for length n (an empty schedule restores the default)."""
    sched = list(schedule)
    arr = (C.c_int * 16)(*sched)
    N.check("mjx_dft_schedule_set", N.lib().mjx_dft_schedule_set(int(n), N.dtype_code(dtype), len(sched), arr,
                                                                 int(tpsm)))
    key = f"dft/{int(n)}/{N.dtype_code(dtype)}"
    if sched:
        _RECORD[key] = {"schedule": sched, "tpsm": int(tpsm)}
        _DFT_DONE.add((int(n), N.dtype_code(dtype)))
    else:
        _RECORD.pop(key, None)
        _DFT_DONE.discard((int(n), N.dtype_code(dtype)))


def autotune_dft(n: int, dtype: torch.dtype = torch.float64, device=None, nrows: Optional[int] = None,
                 reps: int = 5, plan: Optional[torch.Tensor] = None) -> Optional[TuneResult]:
    """Time every candidate schedule x threads per sequence of length n on ``nrows`` rows
    (default: enough for ~4 M complex values, at least 64) and install the fastest.
    Returns None for lengths without a schedule."""
    n = int(n)
    cands = dft_schedule_candidates(n)
    if not cands:
        return None
    N.require_cuda()
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    lib = N.lib()
    code = N.dtype_code(dtype)
    if plan is None:
        plan = torch.empty(lib.mjx_dftn_plan_bytes(n, code), dtype=torch.uint8, device=dev)
        with torch.cuda.device(dev):
            N.check("mjx_dftn_plan_init", lib.mjx_dftn_plan_init(N.ptr(plan), n, code, N.stream_ptr(dev)))
    rows = int(nrows) if nrows else max(64, (1 << 22) // n)
    esz = 8 if dtype == torch.float32 else 16
    scratch = torch.empty(rows * n * esz, dtype=torch.uint8, device=dev)
    times = (C.c_double * 256)()
    ncand, best = C.c_int(), C.c_int()
    with torch.cuda.device(dev):
        N.check("mjx_autotune_dft", lib.mjx_autotune_dft(N.ptr(plan), n, code, rows, N.ptr(scratch),
                                                         scratch.numel(), int(reps), times, 256,
                                                         C.byref(ncand), C.byref(best), N.stream_ptr(dev)))
    tps = []
    for t in (n // 4, n // 8, n // 16):
        t = min(max(t, 1), 256)
        if t not in tps:
            tps.append(t)
    full = [(s, t) for s in cands for t in tps]
    sched, tp = dft_schedule(n, dtype)
    _RECORD[f"dft/{n}/{code}"] = {"schedule": list(sched), "tpsm": tp}
    _DFT_DONE.add((n, code))
    return TuneResult((sched, tp), full[: ncand.value], list(times[: ncand.value]), best.value)


def tune_lengths(lengths: Sequence[Tuple[int, int, torch.Tensor]], dtype: torch.dtype, device) -> None:
    """Tune the DFT lengths of a new plan once per process: (n, rows per transform, plan buffer)."""
    if not enabled():
        return
    _maybe_load_cache()
    code = N.dtype_code(dtype)
    for n, rows, buf in lengths:
        if (int(n), code) in _DFT_DONE or not dft_schedule_candidates(n):
            continue
        autotune_dft(n, dtype, device, nrows=max(64, min(int(rows), (1 << 23) // int(n))), plan=buf)


# ---- stencil tiles ---------------------------------------------------------------

def stencil_rows(ny: int, nx: int, nfields: int, dtype: torch.dtype) -> int:
    """Rows per warp strip installed for this size (0: untuned, the kernel uses 8)."""
    return N.lib().mjx_stencil_rows_get(int(ny), int(nx), int(nfields), N.dtype_code(dtype))


def set_stencil_rows(ny: int, nx: int, nfields: int, dtype: torch.dtype, rows: int) -> None:
    N.check("mjx_stencil_rows_set", N.lib().mjx_stencil_rows_set(int(ny), int(nx), int(nfields),
                                                                 N.dtype_code(dtype), int(rows)))
    key = f"rows/{int(ny)}/{int(nx)}/{int(nfields)}/{N.dtype_code(dtype)}"
    if rows:
        _RECORD[key] = {"rows": int(rows)}
        _STENCIL_DONE.add((int(ny), int(nx), int(nfields), N.dtype_code(dtype)))
    else:
        _RECORD.pop(key, None)


def autotune_stencil(model, dtype: Optional[torch.dtype] = None, reps: int = 5, method: int = 2,
                     device=None) -> TuneResult:
    """Time the stage kernel of ``model`` (an explicit-stepper MOLModel) for strips of
    2, 4, 8, 16 and 32 rows and, for FP32 grids whose rows are a multiple of 4 points,
    the TMA-staged form (64), and install the fastest for its grid size."""
    from moljax_gb300.core.fft_solvers import workspace
    from moljax_gb300.core.stepping import explicit_problem
    N.require_cuda()
    grid = model.grid
    names = model.field_names
    dtype = dtype or model.dtype
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    lib = N.lib()
    code = N.dtype_code(dtype)
    prob = explicit_problem(model, method, t=0.0)
    ws = workspace(lib.mjx_explicit_ws_bytes(grid.ny, grid.nx, len(names), code), dev, "explicit")
    times = (C.c_double * 6)()
    best = C.c_int()
    with torch.cuda.device(dev):
        N.check("mjx_autotune_stencil2d", lib.mjx_autotune_stencil2d(
            C.byref(N.Grid2DC(grid.ny, grid.nx, grid.dy, grid.dx)), code, C.byref(prob), N.ptr(ws), ws.numel(),
            int(reps), times, 6, C.byref(best), N.stream_ptr(dev)))
    tma = dtype == torch.float32 and grid.nx % 4 == 0
    cands = [(r,) for r in ((2, 4, 8, 16, 32, 64) if tma else (2, 4, 8, 16, 32))]
    _RECORD[f"rows/{grid.ny}/{grid.nx}/{len(names)}/{code}"] = {"rows": best.value}
    _STENCIL_DONE.add((grid.ny, grid.nx, len(names), code))
    return TuneResult((best.value,), cands, list(times)[:len(cands)], cands.index((best.value,)))


def tune_stencil_once(model, dtype: torch.dtype) -> None:
    """autotune_stencil on the first use of a grid size in this process (MJX_AUTOTUNE)."""
    if not enabled():
        return
    _maybe_load_cache()
    g = model.grid
    key = (g.ny, g.nx, len(model.field_names), N.dtype_code(dtype))
    if key in _STENCIL_DONE:
        return
    autotune_stencil(model, dtype)


# ---- persistence -----------------------------------------------------------------

def choices() -> Dict[str, dict]:
    """The choices installed through this module in this process."""
    return {k: dict(v) for k, v in _RECORD.items()}


def save(path: str) -> None:
    with open(path, "w") as f:
        json.dump({"format": 1, "choices": choices()}, f, indent=1, sort_keys=True)


def load(path: str) -> int:
    """Install the choices of a saved file; returns how many were installed."""
    with open(path) as f:
        data = json.load(f)
    k = 0
    for key, v in data.get("choices", {}).items():
        parts = key.split("/")
        if parts[0] == "dft" and len(parts) == 3:
            code = int(parts[2])
            set_dft_schedule(int(parts[1]), torch.float32 if code == N.dtype_code(torch.float32) else torch.float64,
                             v["schedule"], v.get("tpsm", 0))
            k += 1
        elif parts[0] == "rows" and len(parts) == 5:
            code = int(parts[4])
            set_stencil_rows(int(parts[1]), int(parts[2]), int(parts[3]),
                             torch.float32 if code == N.dtype_code(torch.float32) else torch.float64, v["rows"])
            k += 1
    return k
