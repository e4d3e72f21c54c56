"""Host wrappers of the native ghost-cell and stencil kernels (``csrc/stencil.cu``).

State dicts hold padded CUDA tensors, exactly as the reference stores them.
Fields of one call are stacked into a contiguous [nfields][ny+2g][nx+2g] block.
"""

from __future__ import annotations

import ctypes as C

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.bc import BCType, side_values


def _bc_arrays(names, bc_spec, grid, t=0.0, params=None):
    kinds = (C.c_int * 4)()
    vals = (C.c_double * 16)()
    for i, name in enumerate(names):
        spec = bc_spec.get(name) if bc_spec else None
        if spec is None:
            kinds[i] = int(BCType.PERIODIC)
            continue
        kinds[i] = int(spec.kind)
        for s, v in enumerate(side_values(spec, grid, t, params)):
            vals[4 * i + s] = v
    return kinds, vals


def stack(state, names):
    """Stacks padded fields into one contiguous tensor (one copy kernel)."""
    return torch.stack([state[n] for n in names]).contiguous()


def pad_interior(interior, grid, bc_spec, names, t=0.0, params=None):
    """[nf][ny][nx] interior -> [nf][ny+2g][nx+2g] with ghosts filled (mjx_bc_pad2d)."""
    N.require_cuda(interior)
    nf = interior.shape[0]
    g = grid.n_ghost
    out = torch.empty((nf, grid.ny + 2 * g, grid.nx + 2 * g), dtype=interior.dtype,
                      device=interior.device)
    kinds, vals = _bc_arrays(names, bc_spec, grid, t, params)
    N.check("mjx_bc_pad2d", N.lib().mjx_bc_pad2d(
        N.ptr(interior), N.ptr(out), nf, grid.ny, grid.nx, g, kinds, vals, grid.dy, grid.dx,
        N.dtype_code(interior.dtype), N.stream_ptr(interior.device)))
    return out


def unpad(padded, grid):
    """[nf][ny+2g][nx+2g] -> contiguous interior [nf][ny][nx] (mjx_unpad2d)."""
    N.require_cuda(padded)
    nf = padded.shape[0]
    out = torch.empty((nf, grid.ny, grid.nx), dtype=padded.dtype, device=padded.device)
    N.check("mjx_unpad2d", N.lib().mjx_unpad2d(
        N.ptr(padded), N.ptr(out), nf, grid.ny, grid.nx, grid.n_ghost,
        N.dtype_code(padded.dtype), N.stream_ptr(padded.device)))
    return out


def apply_bc(state, grid, bc_spec, t=0.0, params=None):
    """moljax/core/bc.py:358-404 on the GPU; fields without a spec pass through."""
    names = [n for n in state if n in bc_spec]
    out = dict(state)
    for i in range(0, len(names), 4):
        chunk = names[i:i + 4]
        src = stack(state, chunk)
        N.require_cuda(src)
        dst = torch.empty_like(src)
        kinds, vals = _bc_arrays(chunk, bc_spec, grid, t, params)
        N.check("mjx_bc_fill2d", N.lib().mjx_bc_fill2d(
            N.ptr(src), N.ptr(dst), len(chunk), grid.ny, grid.nx, grid.n_ghost, kinds, vals,
            grid.dy, grid.dx, N.dtype_code(src.dtype), N.stream_ptr(src.device)))
        for j, n in enumerate(chunk):
            out[n] = dst[j]
    return out


def laplacian_2d(f, grid, coef=1.0):
    """moljax/core/operators.py:311-322: 5-point Laplacian on the interior, ghosts zero."""
    src = f.reshape(1, *f.shape).contiguous()
    N.require_cuda(src)
    dst = torch.empty_like(src)
    c = (C.c_double * 4)(coef, 1.0, 1.0, 1.0)
    N.check("mjx_laplacian2d", N.lib().mjx_laplacian2d(
        N.ptr(src), N.ptr(dst), 1, grid.ny, grid.nx, grid.n_ghost, c, 0, None, None, grid.dy,
        grid.dx, N.dtype_code(src.dtype), N.stream_ptr(src.device)))
    return dst[0]


def model_rhs(state, grid, bc_spec, names, reaction, D, F=0.0, k=0.0, t=0.0, params=None):
    """MOLModel.rhs (moljax/core/model.py:100-118) fused: BCs + D Lap + reaction."""
    src = stack(state, names)
    N.require_cuda(src)
    dst = torch.empty_like(src)
    kinds, vals = _bc_arrays(names, bc_spec, grid, t, params)
    Dc = (C.c_double * 4)(*([float(d) for d in D] + [0.0] * (4 - len(D))))
    N.check("mjx_rhs2d", N.lib().mjx_rhs2d(
        N.ptr(src), N.ptr(dst), len(names), grid.ny, grid.nx, grid.n_ghost, reaction, Dc,
        float(F), float(k), kinds, vals, grid.dy, grid.dx, N.dtype_code(src.dtype),
        N.stream_ptr(src.device)))
    return {n: dst[i] for i, n in enumerate(names)}
