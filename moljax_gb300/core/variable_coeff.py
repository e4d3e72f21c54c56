"""Variable-coefficient diffusion (moljax/core/variable_coeff.py drop-in, the part on the
path): ``apply_variable_diffusion_2d``, one native stencil pass.  The implicit
variable-diffusion solves (the residual and JVP of div((a + b u^c) grad u)) run inside
the Newton-Krylov kernels (``csrc/nk.cu``)."""

from __future__ import annotations

import torch

from moljax_gb300 import _native as N


def apply_variable_diffusion_2d(u: torch.Tensor, D: torch.Tensor, dy: float, dx: float, ng: int, ny: int,
                                nx: int) -> torch.Tensor:
    """div(D grad u) with face averages (D_i + D_{i+1})/2 on the interior of the padded
    field u, ghosts zero (variable_coeff.py:232-287).  D is padded like u, or (ny, nx)
    and then edge-extended."""
    u = u.contiguous()
    N.require_cuda(u)
    if tuple(u.shape) != (ny + 2 * ng, nx + 2 * ng):
        raise ValueError("u must be the padded field (ny + 2 ng, nx + 2 ng)")
    D = torch.as_tensor(D, device=u.device).to(u.dtype).contiguous()
    if tuple(D.shape) == (ny, nx):
        d_int = 1
    elif tuple(D.shape) == tuple(u.shape):
        d_int = 0
    else:
        raise ValueError("D must be (ny, nx) or padded like u")
    out = torch.empty_like(u)
    N.check("mjx_variable_diffusion2d", N.lib().mjx_variable_diffusion2d(
        N.ptr(u), N.ptr(D), d_int, N.ptr(out), int(ny), int(nx), int(ng), float(dy), float(dx),
        N.dtype_code(u.dtype), N.stream_ptr(u.device)))
    return out


def apply_variable_diffusion_1d(u: torch.Tensor, D: torch.Tensor, dx: float, ng: int, n: int) -> torch.Tensor:
    """d/dx(D du/dx) with face averages on the interior of a padded 1D field, ghosts zero
    (variable_coeff.py:189-229): the 2D kernel on 2 ng + 1 identical rows, whose y fluxes
    vanish."""
    u = torch.as_tensor(u)
    D = torch.as_tensor(D, device=u.device).to(u.dtype)
    rows = 2 * ng + 1
    u2 = u.reshape(1, -1).expand(rows, -1).contiguous()
    if D.shape[-1] == n:
        D2 = D.reshape(1, -1).expand(1, -1).contiguous()
    else:
        D2 = D.reshape(1, -1).expand(rows, -1).contiguous()
    return apply_variable_diffusion_2d(u2, D2, 1.0, dx, ng, 1, n)[ng].clone()
