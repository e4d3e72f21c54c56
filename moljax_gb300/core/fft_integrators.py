"""Exponential time differencing on periodic grids (moljax/core/fft_integrators.py).

``etdrk4_gray_scott`` runs the coupled Gray-Scott ETDRK4 of the reference
benchmark (benchmarks/benchmark_gray_scott.py:336-417) natively: contour-
integral coefficients in FP64 on the GPU, FP32 or FP64 state, 8 fused kernels
per step replayed from a CUDA graph.  ``etdrk4_step`` keeps the library
signature (fft_integrators.py:252-341) for models whose nonlinear part is a
native reaction; the reference library applies the later stages per field and
cannot couple u and v (fft_integrators.py:311-327), this implementation couples
them as the benchmark does.
"""

from __future__ import annotations

import ctypes as C
import torch

from moljax_gb300 import _native as N
from moljax_gb300.core import stencil
from moljax_gb300.core.fft_solvers import get_plan, workspace

_coeff_key = {}


def _symbol_code(symbol):
    return {"fd": N.SYMBOL_FD, "spectral": N.SYMBOL_SPECTRAL}[symbol]


def etdrk4_gray_scott(model, y0, dt: float, n_steps: int, symbol: str = "fd",
                      variant: str = "cox-matthews"):
    """Fixed-step coupled ETDRK4 on a Gray-Scott MOLModel (padded state in and out).

    ``variant="cox-matthews"`` is the fourth-order method (the library's
    coefficients, fft_integrators.py:106-113); ``variant="benchmark"``
    reproduces benchmarks/benchmark_gray_scott.py:415, whose final update uses
    f2 (N^a + N^b) without the factor 2 of the Kassam-Trefethen form.
    """
    f2_factor = {"cox-matthews": 2.0, "benchmark": 1.0}[variant]
    if model.reaction_kind != N.REACT_GRAY_SCOTT:
        raise NotImplementedError("native ETDRK4 is built for the coupled Gray-Scott reaction")
    grid = model.grid
    names = model.field_names
    interior = stencil.unpad(stencil.stack(y0, names), grid)
    D = model.diffusivities()
    ny, nx = grid.ny, grid.nx
    plan = get_plan(ny, nx, grid.dy, grid.dx, symbol, interior.dtype, interior.device)
    lib = N.lib()
    ws = workspace(lib.mjx_etdrk4_ws_bytes(ny, nx, plan.code), plan.device, "etd")
    key = (ny, nx, grid.dy, grid.dx, symbol, interior.dtype, D["u"], D["v"], float(dt), f2_factor,
           ws.data_ptr())
    recompute = int(_coeff_key.get(str(plan.device)) != key)
    _coeff_key[str(plan.device)] = key
    out = torch.empty_like(interior)
    Dc = (C.c_double * 2)(D["u"], D["v"])
    N.check("mjx_etdrk4_gray_scott2d", lib.mjx_etdrk4_gray_scott2d(
        N.ptr(plan.buf), C.byref(plan.cgrid), plan.code, _symbol_code(symbol), Dc,
        float(model.params["F"]), float(model.params["k"]), float(dt), f2_factor, int(n_steps),
        N.ptr(interior), N.ptr(out), N.ptr(ws), ws.numel(), recompute,
        N.stream_ptr(plan.device)))
    padded = stencil.pad_interior(out, grid, model.bc_spec, names)
    return {n: padded[i] for i, n in enumerate(names)}


def etdrk4_step(state, t: float, dt: float, linear_ops, nonlinear_rhs, model=None):
    """One ETDRK4 step (fft_integrators.py:252-341).

    ``linear_ops`` maps field names to ``DiffusionOperator``; ``nonlinear_rhs``
    must be the model's native Gray-Scott reaction (a MOLModel, or a
    NonlinearOp carrying kind MJX_REACT_GRAY_SCOTT together with ``model=``).
    """
    m = model if model is not None else nonlinear_rhs
    if not hasattr(m, "reaction_kind"):
        raise NotImplementedError("etdrk4_step runs natively for a Gray-Scott MOLModel")
    return etdrk4_gray_scott(m, state, dt, 1)


def etd_integrate(model, y0, t0: float, t_end: float, dt: float, symbol: str = "fd",
                  variant: str = "cox-matthews"):
    """Fixed-step ETDRK4 from t0 to t_end, n = ceil((t_end-t0)/dt) steps
    (fft_integrators.py:344-393; step count as benchmark_gray_scott.py)."""
    import math
    n = int(math.ceil((t_end - t0) / dt - 1e-12))
    return etdrk4_gray_scott(model, y0, dt, n, symbol, variant), t0 + n * dt
