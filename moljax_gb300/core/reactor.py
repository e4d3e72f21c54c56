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
RK4_DANCKWERTS, RK4_ROBIN, RK4_NEUMANN = 3, 4, 5
RK4_VARIANTS = {"danckwerts": RK4_DANCKWERTS, "robin": RK4_ROBIN, "neumann": RK4_NEUMANN}


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
    """All cases in one launch; returns a list of final concentration profiles.  Cases of
    the penalty-RK4 variants (RK4_*) go through ``mjx_reactor_rk4_batch`` (all cases of
    one call must then be RK4 ones), the others through ``mjx_reactor_cn_batch``."""
    if not cases:
        return []
    rk4 = [c.variant >= RK4_DANCKWERTS for c in cases]
    if any(rk4) and not all(rk4):
        raise ValueError("solve_batch: RK4 and CN reactor cases go in separate batches")
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
    entry = "mjx_reactor_rk4_batch" if rk4[0] else "mjx_reactor_cn_batch"
    N.check(entry, getattr(N.lib(), entry)(
        N.ptr(inst), len(cases), max(c.n for c in cases), N.dtype_code(dtype), N.ptr(out), s))
    res = [out[offs[i]:offs[i] + c.n] for i, c in enumerate(cases)]
    return res


def tubular_reactor_cn(n: int, Pe: float, Da: float, dt: float, n_steps: int,
                       variant: str = "danckwerts", c_init: float = 1.0, dtype=torch.float64):
    """One solve (solve_reactor_cn_jit / run_reactor_cn semantics)."""
    v = DANCKWERTS if variant == "danckwerts" else DIRICHLET
    return solve_batch([ReactorCase(n, Pe, Da, dt, n_steps, v, c_init)], dtype)[0]


def tubular_rk4_dt(n: int, Pe: float, t_final: float):
    """dt = min(0.5 dz, 0.25 Pe dz^2, 0.01), n_steps = int(t_final / dt), dz = 1/(n-1)
    (benchmarks/benchmark_tubular_reactor.py:283-286)."""
    dz = 1.0 / (n - 1)
    dt = min(0.5 * dz, 0.25 * Pe * dz ** 2, 0.01)
    return dt, int(t_final / dt)


def tubular_rk4_case(Pe: float, Da: float, bc_type: str, N: int = 128, t_final: float = 10.0,
                     c_in: float = 1.0) -> ReactorCase:
    """The case ``run_single_benchmark(Pe, Da, bc_type, N, t_final)`` of
    benchmarks/benchmark_tubular_reactor.py:254-301 runs: zeros (Danckwerts, Robin) or ones
    (Neumann) at t = 0, the CFL step, RK4 to t_final."""
    if bc_type not in RK4_VARIANTS:
        raise ValueError(f"Unknown BC type: {bc_type}")
    dt, n_steps = tubular_rk4_dt(N, Pe, t_final)
    return ReactorCase(N, Pe, Da, dt, n_steps, RK4_VARIANTS[bc_type],
                       1.0 if bc_type == "neumann" else 0.0, c_in)


def reactor_summary(c: torch.Tensor, Pe: float, Da: float, bc_type: str, t_final: float):
    """conversion (1 - outlet; the mean for Neumann), max error against the analytic
    profile (Danckwerts steady state, or e^{-Da t} for Neumann) and the outlet value
    (benchmarks/benchmark_tubular_reactor.py:207-235, 294-296), computed on the host in FP64."""
    import numpy as np
    c = c.detach().double().cpu().numpy()
    n = c.shape[-1]
    z = np.linspace(0, 1, n)
    if bc_type == "neumann":
        ref = np.exp(-Da * t_final) * np.ones(n)
        conv = float(c.mean())
    else:
        disc = Pe ** 2 + 4 * Pe * Da
        r1, r2 = (Pe + np.sqrt(disc)) / 2, (Pe - np.sqrt(disc)) / 2
        a, b = np.linalg.solve(np.array([[r1 / Pe - 1, r2 / Pe - 1], [r1 * np.exp(r1), r2 * np.exp(r2)]]),
                               np.array([-1.0, 0.0]))
        ref = a * np.exp(r1 * z) + b * np.exp(r2 * z)
        conv = float(1.0 - c[-1])
    return {"conversion": conv, "error": float(np.max(np.abs(c - ref))), "final_outlet_c": float(c[-1])}


def run_tubular_sweep(bc_types=("danckwerts", "robin", "neumann"), Pe_values=(1, 10, 100),
                      Da_values=(0.1, 1, 10), N: int = 128, t_final: float = 15.0, dtype=torch.float64,
                      device="cuda"):
    """Every (BC, Pe, Da) case of run_full_sweep (benchmarks/benchmark_tubular_reactor.py:304-329)
    in one launch; returns {"<bc>_Pe<Pe>_Da<Da>": summary + dt + n_steps}."""
    keys, cases = [], []
    for bc in bc_types:
        for Pe in Pe_values:
            for Da in Da_values:
                keys.append((bc, Pe, Da))
                cases.append(tubular_rk4_case(Pe, Da, bc, N, t_final))
    outs = solve_batch(cases, dtype, device)
    res = {}
    for (bc, Pe, Da), case, c in zip(keys, cases, outs):
        r = reactor_summary(c, Pe, Da, bc, t_final)
        r.update(bc_type=bc, Pe=Pe, Da=Da, dt=case.dt, n_steps=case.n_steps)
        res[f"{bc}_Pe{Pe}_Da{Da}"] = r
    return res
