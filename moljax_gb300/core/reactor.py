"""Tubular reactor with Danckwerts/Dirichlet inlet, Crank-Nicolson (batched, native).

The reference computes these in its benchmark scripts with dense O(n^2)
operators (benchmarks/benchmark_reactor_vs_diffrax.py:40-138,
benchmarks/benchmark_method_comparison.py:56-160).  Here many solves of
different n / Pe / Da / dt run in one launch (``mjx_reactor_cn_batch``), one
CTA per solve with the whole time loop in shared memory.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Sequence

import torch

from moljax_gb300 import _native as N

DANCKWERTS, DIRICHLET, DANCKWERTS_CN = 0, 1, 2


@dataclass
class ReactorCase:
    n: int
    Pe: float
    Da: float
    dt: float
    n_steps: int
    variant: int = DANCKWERTS
    c_init: float = 0.0
    c_inlet: float = 1.0


def served_dt(n: int, t_final: float = 5.0):
    """dt = min(10 dz, 0.05, t_final/100), dz = 1/(n-1) (benchmark_method_comparison.py:215-217)."""
    dz = 1.0 / (n - 1)
    dt = min(10 * dz, 0.05, t_final / 100)
    return dt, int(t_final / dt)


def solve_batch(cases: Sequence[ReactorCase], dtype=torch.float32, device="cuda", stream=None):
    """All cases in one launch; returns a list of final concentration profiles."""
    if not cases:
        return []
    offs, o = [], 0
    arr = (N.ReactorInstanceC * len(cases))()
    for i, c in enumerate(cases):
        arr[i] = N.ReactorInstanceC(c.n, c.variant, c.n_steps, 0, o, c.Pe, c.Da, c.dt, c.c_init,
                                    c.c_inlet)
        offs.append(o)
        o += c.n
    dev = torch.device(device)
    raw = torch.frombuffer(bytearray(C.string_at(arr, C.sizeof(arr))), dtype=torch.uint8)
    inst = raw.to(dev, non_blocking=False)
    out = torch.empty(o, dtype=dtype, device=dev)
    s = C.c_void_p(stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream)
    N.check("mjx_reactor_cn_batch", N.lib().mjx_reactor_cn_batch(
        N.ptr(inst), len(cases), max(c.n for c in cases), N.dtype_code(dtype), N.ptr(out), s))
    res = [out[offs[i]:offs[i] + c.n] for i, c in enumerate(cases)]
    return res


def tubular_reactor_cn(n: int, Pe: float, Da: float, dt: float, n_steps: int,
                       variant: str = "danckwerts", c_init: float = 1.0, dtype=torch.float64):
    """One solve (solve_reactor_cn_jit / run_reactor_cn semantics)."""
    v = DANCKWERTS if variant == "danckwerts" else DIRICHLET
    return solve_batch([ReactorCase(n, Pe, Da, dt, n_steps, v, c_init)], dtype)[0]
