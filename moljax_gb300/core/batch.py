"""Batched adaptive IMEX-Strang: many Gray-Scott solves in one native engine.

The reference batches only by stacking arrays of one shape under ``vmap``
(moljax/core/jit_kernels.py:422-441, 481-531; fft_integrators.py:473-510), and
each ``adaptive_integrate_imex`` call (moljax/core/stepping.py:1146-1371) runs
its own ``lax.while_loop``.  Here solves of different grid sizes, parameters
and time spans share one engine (``mjx_gsbatch_*``): every attempt stage is
one kernel launch over all solves in flight, each solve keeps its own dt,
controller state, accept mask, status and t/dt history on the device, and the
attempt loop is a CUDA graph with a conditional while node.  Each solve runs
the mixed-precision attempt of ``adaptive_integrate_imex(precision="mixed")``
(float-float spectral state, FP32 increment transforms).

``GrayScottBatch`` is the engine (admit / run / retire, for continuous
batching); ``adaptive_integrate_imex_batch`` solves a list of problems.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence

import numpy as np
import torch

from moljax_gb300 import _native as N
from moljax_gb300.core import stencil
from moljax_gb300.core.dt_policy import CFLParams, PIDParams, imex_cfl_dt
from moljax_gb300.core.stepping import AdaptiveResult, _pid_c


@dataclass
class GrayScottProblem:
    """One Gray-Scott solve: grid (periodic Grid2D), parameters, initial state
    (padded StateDict {"u", "v"} or interior tensor (2, ny, nx)) and time span."""
    grid: object
    Du: float
    Dv: float
    F: float
    k: float
    y0: object
    t0: float = 0.0
    t_end: float = 1.0
    dt0: float = 1.0
    pid: Optional[PIDParams] = None
    cfl: Optional[CFLParams] = None
    max_steps: int = 10000
    save_every: int = 1
    max_attempts: int = 0


def _interior(y0, grid, dtype, device):
    if isinstance(y0, dict):
        x = stencil.unpad(stencil.stack(y0, ("u", "v")), grid)
    else:
        x = torch.as_tensor(y0)
    x = x.to(device=device, dtype=dtype).contiguous()
    if tuple(x.shape) != (2, grid.ny, grid.nx):
        raise ValueError(f"initial state must be (2, {grid.ny}, {grid.nx}) or a padded (u, v) StateDict")
    return x


class GrayScottBatch:
    """Continuous-batching engine for adaptive Gray-Scott IMEX-Strang solves.

    ``admit`` places a solve in a free slot (its workspace comes from the torch
    allocator, sized by ``mjx_gsbatch_instance_bytes``), ``run`` advances every
    running solve until an epoch ends, ``finished`` lists the slots that are done
    and ``retire`` returns a finished solve's final state and result and frees its
    slot.  ``request_stop`` (any thread) ends a running epoch at its next attempt
    boundary.  One thread drives an engine.
    """

    def __init__(self, device=None, max_instances: int = 256, max_work: Optional[int] = None):
        N.require_cuda()
        self.device = torch.device(device or "cuda")
        lib = N.lib()
        if max_work is None:  # room for max_instances solves of 512^2
            max_work = max_instances * lib.mjx_gsbatch_work_items(512, 512)
        self.max_instances = int(max_instances)
        self.max_work = int(max_work)
        nbytes = lib.mjx_gsbatch_bytes(self.max_instances, self.max_work)
        if nbytes == 0:
            raise ValueError("bad engine capacity")
        self._ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check("mjx_gsbatch_create", lib.mjx_gsbatch_create(C.byref(h), self.max_instances, self.max_work,
                                                                 N.ptr(self._ws), nbytes))
        self._h = h
        self._slots: Dict[int, dict] = {}
        self.work_items = 0

    # -------------------------------------------------------------- admission
    def fits(self, ny: int, nx: int) -> bool:
        """True when a solve of this size has a free slot and work-list room now."""
        w = N.lib().mjx_gsbatch_work_items(ny, nx)
        return w > 0 and len(self._slots) < self.max_instances and self.work_items + w <= self.max_work

    @staticmethod
    def instance_bytes(ny: int, nx: int, max_steps: int = 10000, save_every: int = 1) -> int:
        return int(N.lib().mjx_gsbatch_instance_bytes(ny, nx, max_steps // save_every + 1))

    def admit(self, p: GrayScottProblem, stream=None) -> int:
        grid = p.grid
        io = p.y0["u"].dtype if isinstance(p.y0, dict) else torch.as_tensor(p.y0).dtype
        if io not in (torch.float32, torch.float64):
            io = torch.float64
        y0 = _interior(p.y0, grid, io, self.device)
        pid = p.pid or PIDParams()
        cfl = p.cfl or CFLParams()
        d = N.GsInstanceC()
        d.ny, d.nx, d.dy, d.dx = grid.ny, grid.nx, grid.dy, grid.dx
        d.Du, d.Dv, d.F, d.k = float(p.Du), float(p.Dv), float(p.F), float(p.k)
        d.t0, d.t_end, d.dt0 = float(p.t0), float(p.t_end), float(p.dt0)
        d.dt_cfl = imex_cfl_dt(grid, {"Du": p.Du, "Dv": p.Dv, "F": p.F, "k": p.k}, cfl)
        d.max_steps, d.save_every, d.max_attempts = int(p.max_steps), int(p.save_every), int(p.max_attempts)
        d.pid = _pid_c(pid)
        nbytes = self.instance_bytes(grid.ny, grid.nx, p.max_steps, p.save_every)
        if nbytes == 0:
            raise ValueError(f"grid {grid.ny}x{grid.nx}: the batch takes powers of two, 16 <= ny <= 2048, "
                             "16 <= nx <= 4096")
        ws = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
        slot = C.c_int(-1)
        s = stream if stream is not None else N.stream_ptr(self.device)
        with torch.cuda.device(self.device):
            N.check("mjx_gsbatch_admit", N.lib().mjx_gsbatch_admit(
                self._h, C.byref(d), N.dtype_code(io), N.ptr(y0), N.ptr(ws), nbytes, C.byref(slot), s))
        w = N.lib().mjx_gsbatch_work_items(grid.ny, grid.nx)
        self._slots[slot.value] = {"ws": ws, "grid": grid, "io": io, "work": w,
                                   "max_saves": p.max_steps // p.save_every + 1}
        self.work_items += w
        return slot.value

    # -------------------------------------------------------------- epochs
    def run(self, max_attempts: int = 1 << 30, stop_after_finished: int = 0, stream=None):
        """Runs one epoch; returns (solves still running, finished solves awaiting retire)."""
        nr, nf = C.c_int(0), C.c_int(0)
        s = stream if stream is not None else N.stream_ptr(self.device)
        with torch.cuda.device(self.device):
            N.check("mjx_gsbatch_run", N.lib().mjx_gsbatch_run(self._h, int(max_attempts), int(stop_after_finished),
                                                              C.byref(nr), C.byref(nf), s))
        return nr.value, nf.value

    def finished(self) -> List[int]:
        cap = max(1, len(self._slots))
        arr = (C.c_int * cap)()
        n = C.c_int(0)
        N.check("mjx_gsbatch_finished", N.lib().mjx_gsbatch_finished(self._h, arr, cap, C.byref(n)))
        return [arr[i] for i in range(min(n.value, cap))]

    def retire(self, slot: int, dtype=None, stream=None):
        """Final state (interior tensor (2, ny, nx)) and AdaptiveResult of a finished solve."""
        meta = self._slots[slot]
        grid = meta["grid"]
        dt = dtype or meta["io"]
        out = torch.empty((2, grid.ny, grid.nx), dtype=dt, device=self.device)
        res = N.AdaptiveResultC()
        s = stream if stream is not None else N.stream_ptr(self.device)
        ns = meta["max_saves"]
        ht = np.zeros(ns, dtype=np.float64)
        hdt = np.zeros(ns, dtype=np.float64)
        dp = C.POINTER(C.c_double)
        with torch.cuda.device(self.device):
            st = N.lib().mjx_gsbatch_retire(self._h, slot, N.dtype_code(dt), N.ptr(out), ht.ctypes.data_as(dp),
                                            hdt.ctypes.data_as(dp), C.byref(res), s)
        N.check("mjx_gsbatch_retire", st)
        self.work_items -= meta["work"]
        del self._slots[slot]
        r = AdaptiveResult(res.t_final, {"u": out[0], "v": out[1]}, torch.from_numpy(ht), None,
                           torch.from_numpy(hdt), res.n_saved, res.n_accepted, res.n_rejected, res.status)
        return out, r

    def request_stop(self, stop: bool = True):
        N.lib().mjx_gsbatch_request_stop(self._h, 1 if stop else 0)

    @property
    def n_in_flight(self) -> int:
        return len(self._slots)

    def close(self):
        if self._h is not None and self._h.value:
            N.lib().mjx_gsbatch_destroy(self._h)
            self._h = None
            self._slots.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


def adaptive_integrate_imex_batch(problems: Sequence[GrayScottProblem], device=None,
                                  dtype=torch.float32, max_instances: Optional[int] = None):
    """Solves every problem in one batch engine (all admitted at once, then epochs
    until all finish); returns a list of (final interior state (2, ny, nx),
    AdaptiveResult) in the order of ``problems``.  Each result is the
    mixed-precision ``adaptive_integrate_imex`` solve of that problem alone."""
    dev = torch.device(device or "cuda")
    eng = GrayScottBatch(dev, max_instances=max_instances or max(1, len(problems)),
                         max_work=sum(N.lib().mjx_gsbatch_work_items(p.grid.ny, p.grid.nx) for p in problems) or 1)
    try:
        slots = [eng.admit(p) for p in problems]
        out: Dict[int, tuple] = {}
        while len(out) < len(problems):
            eng.run()
            for s in eng.finished():
                out[s] = eng.retire(s, dtype)
        return [out[s] for s in slots]
    finally:
        eng.close()
