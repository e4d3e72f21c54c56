"""PDE model assembly (moljax/core/model.py drop-in).

``MOLModel`` keeps the reference fields (grid, bc_spec, params, linear_ops,
nonlinear_ops, metadata; model.py:34-118).  ``rhs`` runs the fused native
kernel (BCs + D Lap + reaction) when the model was built by a factory below.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Dict, List, Optional, Tuple

import torch

from moljax_gb300 import _native as N
from moljax_gb300.core.bc import BCType, FieldBCSpec
from moljax_gb300.core.grid import Grid2D
from moljax_gb300.core.operators import LinearOp, NonlinearOp, gray_scott_reaction_op, \
    fisher_kpp_reaction_op


@dataclass(frozen=True)
class MOLModel:
    grid: Any
    bc_spec: Dict[str, FieldBCSpec]
    params: Dict[str, Any]
    linear_ops: Tuple[LinearOp, ...] = field(default_factory=tuple)
    nonlinear_ops: Tuple[NonlinearOp, ...] = field(default_factory=tuple)
    metadata: Dict[str, Any] = field(default_factory=dict)

    @property
    def dtype(self) -> torch.dtype:
        return self.params.get("dtype", torch.float64)

    @property
    def field_names(self) -> List[str]:
        return list(self.bc_spec.keys())

    # native description of the model: (reaction id, per-field diffusivities)
    @property
    def reaction_kind(self) -> int:
        kinds = [op.kind for op in self.nonlinear_ops]
        if not kinds:
            return N.REACT_NONE
        if len(kinds) != 1 or kinds[0] is None:
            raise NotImplementedError(
                "fused GPU drivers support one built-in reaction (Gray-Scott or Fisher-KPP); "
                f"got {[op.name for op in self.nonlinear_ops]}")
        return kinds[0]

    def diffusivities(self) -> Dict[str, float]:
        if "diffusivities" in self.metadata:
            return dict(self.metadata["diffusivities"])
        out = {}
        for n in self.field_names:
            out[n] = float(self.params.get(f"D{n}", self.params.get("D", 0.0)))
        return out

    def apply_bcs(self, state, t: float = 0.0):
        from moljax_gb300.core import stencil
        return stencil.apply_bc(state, self.grid, self.bc_spec, t, self.params)

    def rhs(self, state, t: float = 0.0):
        """apply_bcs -> D Lap + reaction, fused in one kernel (model.py:100-118)."""
        from moljax_gb300.core import stencil
        if self.metadata.get("kind") == "vardiff":
            return _vardiff_rhs(self, state)
        if self.metadata.get("advection"):
            return _explicit_rhs(self, state, t)
        D = self.diffusivities()
        names = self.field_names
        rx = self.reaction_kind
        F = self.params.get("r", 1.0) if rx == N.REACT_FISHER else self.params.get("F", 0.0)
        return stencil.model_rhs(state, self.grid, self.bc_spec, names, rx,
                                 [D[n] for n in names], F, self.params.get("k", 0.0), t,
                                 self.params)

    def create_initial_state(self, init_fns=None, fill_values=None, device="cuda"):
        init_fns = init_fns or {}
        fill_values = fill_values or {}
        g = self.grid
        shape = (g.ny_total, g.nx_total)
        out = {}
        for n in self.field_names:
            if n in init_fns:
                X, Y = g.meshgrid(include_ghost=True)
                out[n] = torch.as_tensor(init_fns[n](X, Y)).to(device=device, dtype=self.dtype)
            else:
                out[n] = torch.full(shape, float(fill_values.get(n, 0.0)), dtype=self.dtype,
                                    device=device)
        return out


def create_gray_scott_model(grid: Grid2D, Du: float = 0.16, Dv: float = 0.08, F: float = 0.04,
                            k: float = 0.06, bc_type: BCType = BCType.PERIODIC,
                            dtype: torch.dtype = torch.float64) -> MOLModel:
    """moljax/core/model.py:213-292."""
    from moljax_gb300.core import stencil
    bc_spec = {"u": FieldBCSpec(kind=bc_type), "v": FieldBCSpec(kind=bc_type)}
    params = {"Du": Du, "Dv": Dv, "F": F, "k": k, "dtype": dtype}

    def diffusion_apply(state, grid, t, params):
        return {"u": stencil.laplacian_2d(state["u"], grid, params["Du"]),
                "v": stencil.laplacian_2d(state["v"], grid, params["Dv"])}

    def diffusion_dt_bound(grid, params):
        return 0.25 * grid.min_dx2 / (max(params["Du"], params["Dv"]) + 1e-14)

    diffusion = LinearOp("gray_scott_diffusion", diffusion_apply, diffusion_dt_bound, "diffusion")
    return MOLModel(grid, bc_spec, params, (diffusion,), (gray_scott_reaction_op(),),
                    {"field_names": ["u", "v"], "pde_type": "reaction_diffusion", "stiff": True,
                     "diffusivities": {"u": Du, "v": Dv}})


def create_gray_scott_periodic_fft(grid: Grid2D, Du: float = 0.16, Dv: float = 0.08,
                                   F: float = 0.04, k: float = 0.06,
                                   dtype: torch.dtype = torch.float64, device=None):
    """moljax/core/model.py:529-584 -> (model, fft_cache, diffusivities)."""
    from moljax_gb300.core.fft_solvers import create_fft_cache
    model = create_gray_scott_model(grid, Du, Dv, F, k, BCType.PERIODIC, dtype)
    cache = create_fft_cache(grid, dtype, device)
    diff = {"u": Du, "v": Dv}
    md = dict(model.metadata)
    md.update(fft_cache=cache, diffusivities=diff, supports_fft=True)
    return MOLModel(model.grid, model.bc_spec, model.params, model.linear_ops,
                    model.nonlinear_ops, md), cache, diff


def gray_scott_factory(nx: int = 256, ny: Optional[int] = None, Du: float = 2e-5,
                       Dv: float = 1e-5, F: float = 0.035, k: float = 0.065, L: float = 2.5,
                       dtype: torch.dtype = torch.float32, device=None) -> MOLModel:
    """README.md:65-73 factory: periodic Gray-Scott on [0, L]^2 with its FFT cache."""
    grid = Grid2D(nx, ny or nx, 0.0, L, 0.0, L)
    model, _, _ = create_gray_scott_periodic_fft(grid, Du, Dv, F, k, dtype, device)
    return model


def create_fisher_kpp_model(grid: Grid2D, D: float = 0.01, r: float = 1.0,
                            bc_type: BCType = BCType.PERIODIC,
                            dtype: torch.dtype = torch.float64) -> MOLModel:
    """moljax/core/model.py:470-524 (D Lap u + r u (1-u))."""
    from moljax_gb300.core import stencil
    params = {"D": D, "r": r, "dtype": dtype}

    def diffusion_apply(state, grid, t, params):
        return {"u": stencil.laplacian_2d(state["u"], grid, params["D"])}

    diffusion = LinearOp("fisher_diffusion", diffusion_apply, None, "diffusion")
    return MOLModel(grid, {"u": FieldBCSpec(kind=bc_type)}, params, (diffusion,),
                    (fisher_kpp_reaction_op("u", "r"),),
                    {"field_names": ["u"], "diffusivities": {"u": D}})


def create_advection_diffusion_model(grid: Grid2D, field_names=("c1", "c2"), D: float = 0.01,
                                     vx: float = 1.0, vy: float = 0.0,
                                     bc_type: BCType = BCType.PERIODIC, use_upwind: bool = True,
                                     dtype: torch.dtype = torch.float64,
                                     reactions: Optional[NonlinearOp] = None) -> MOLModel:
    """dc_i/dt = D Lap(c_i) - vx dc_i/dx - vy dc_i/dy (moljax/core/model.py:295-370).

    The operator is one linear op, as in the reference (upwind d1_upwind_2d or
    central differences); the explicit steppers evaluate it in fused native kernels.
    ``reactions`` (an extension of the reference signature): a native reaction op of the
    species, e.g. ``make_kinetics_op``, added to the model's nonlinear ops.
    """
    names = list(field_names)
    bc_spec = {n: FieldBCSpec(kind=bc_type) for n in names}
    params = {"D": D, "vx": vx, "vy": vy, "dtype": dtype}

    def advdiff_apply(state, g, t, p):
        return _explicit_rhs_raw(state, g, bc_spec, names, p, 1 if use_upwind else 2, t)

    def advdiff_dt_bound(g, p):  # model.py:358-369
        vmax = abs(p["vx"]) + abs(p["vy"])
        return min(g.min_dx / (vmax + 1e-14), 0.25 * g.min_dx2 / (p["D"] + 1e-14))

    op = LinearOp("advection_diffusion", advdiff_apply, advdiff_dt_bound, "advection_diffusion")
    if reactions is not None and reactions.native is not None and list(reactions.native[0]) != names:
        raise ValueError("the reaction network's species must be the model's fields, in order")
    return MOLModel(grid, bc_spec, params, (op,), (reactions,) if reactions is not None else (),
                    {"field_names": names, "pde_type": "advection_diffusion",
                     "advection": 1 if use_upwind else 2,
                     "diffusivities": {n: D for n in names}})


def create_advdiff_periodic_fft(grid: Grid2D, field_names=("c1", "c2"), D: float = 0.01,
                                vx: float = 1.0, vy: float = 0.0, use_upwind: bool = True,
                                dtype: torch.dtype = torch.float64, device=None):
    """moljax/core/model.py:587-642 -> (model, fft_cache, diffusivities)."""
    from moljax_gb300.core.fft_solvers import create_fft_cache
    model = create_advection_diffusion_model(grid, field_names, D, vx, vy, BCType.PERIODIC,
                                             use_upwind, dtype)
    cache = create_fft_cache(grid, dtype, device)
    diff = {n: D for n in model.field_names}
    md = dict(model.metadata)
    md.update(fft_cache=cache, diffusivities=diff, supports_fft=True)
    return MOLModel(model.grid, model.bc_spec, model.params, model.linear_ops,
                    model.nonlinear_ops, md), cache, diff


def _explicit_rhs_raw(state, grid, bc_spec, names, params, advection, t=0.0):
    proto = MOLModel(grid, bc_spec, params, (), (), {"advection": advection,
                                                    "diffusivities": {n: params["D"] for n in names}})
    return _explicit_rhs(proto, state, t)


def _explicit_rhs(model: MOLModel, state, t):
    """MOLModel.rhs through the explicit stage kernel (BCs on the fly, ghosts of the result zero)."""
    import ctypes as C
    from moljax_gb300.core import stencil
    from moljax_gb300.core.stepping import explicit_problem
    names = model.field_names
    prob = explicit_problem(model, 2, t=t)
    interior = stencil.unpad(stencil.stack(state, names), model.grid)
    N.require_cuda(interior)
    out = torch.empty_like(interior)
    g = model.grid
    N.check("mjx_explicit_rhs2d", N.lib().mjx_explicit_rhs2d(
        C.byref(N.Grid2DC(g.ny, g.nx, g.dy, g.dx)), N.dtype_code(interior.dtype), C.byref(prob),
        N.ptr(interior), N.ptr(out), N.stream_ptr(interior.device)))
    res = {}
    for i, n in enumerate(names):
        padded = torch.zeros_like(state[n])
        padded[g.interior_slice] = out[i]
        res[n] = padded
    return res


def create_variable_diffusion_model(grid: Grid2D, a: float = 1.0, b: float = 1.0, c: float = 1.0,
                                    dtype: torch.dtype = torch.float64) -> MOLModel:
    """u_t = div((a + b u^2) grad u) - c u^3 with homogeneous Dirichlet ghosts.

    The nonlinear-diffusion model of the Newton-Krylov workload: the flux is the
    face-averaged conservative form of apply_variable_diffusion_2d
    (moljax/core/variable_coeff.py:232-287) with D = a + b u^2 evaluated on the
    ghost-filled state, minus the reaction c u^3.  Square grids (n x n, n a power
    of two <= 2048) on any spacing.  The implicit steppers (be_step, cn_step,
    bdf2_step, integrate_fixed_dt, adaptive_integrate with BE/CN/BDF2) run this
    model on the native Newton-Krylov solver.
    """
    if grid.nx != grid.ny:
        raise NotImplementedError("the native variable-diffusion model needs nx == ny")
    bc_spec = {"u": FieldBCSpec(kind=BCType.DIRICHLET)}
    params = {"a": a, "b": b, "c": c, "dtype": dtype}
    op = NonlinearOp("variable_diffusion_reaction", lambda st, g, tt, pp: _vardiff_rhs_raw(
        st, g, pp), None)
    return MOLModel(grid, bc_spec, params, (), (op,),
                    {"field_names": ["u"], "kind": "vardiff", "abc": (a, b, c), "stiff": True})


def _vardiff_rhs_raw(state, grid, params):
    import ctypes as C
    from moljax_gb300.core import stencil
    u = state["u"]
    N.require_cuda(u)
    interior = stencil.unpad(u[None], grid)[0].to(torch.float64).contiguous()
    out = torch.empty_like(interior)
    abc = (C.c_double * 3)(params["a"], params["b"], params["c"])
    N.check("mjx_vardiff_rhs2d", N.lib().mjx_vardiff_rhs2d(
        grid.nx, float(grid.dy), float(grid.dx), abc, N.ptr(interior), N.ptr(out),
        N.stream_ptr(u.device)))
    padded = torch.zeros_like(u, dtype=torch.float64)
    padded[grid.interior_slice] = out
    return {"u": padded.to(u.dtype)}


def vardiff_jvp(model: MOLModel, u, v, a0: float = 0.0, beta: float = -1.0):
    """a0 v - beta J_F(u) v for the variable-diffusion model, with the hand-written native
    JVP (``mjx_vardiff_jvp2d``): J_F(u) v by default, the JVP of an implicit residual
    a0 y + cst - beta F(y) otherwise (moljax/core/newton_krylov.py:61-80 takes it with
    jax.jvp).  u, v: interior (n, n) tensors; FP64 result."""
    import ctypes as C
    grid = model.grid
    N.require_cuda(u, v)
    u64, v64 = u.to(torch.float64).contiguous(), v.to(torch.float64).contiguous()
    out = torch.empty_like(u64)
    a, b, c = model.metadata["abc"]
    abc = (C.c_double * 3)(a, b, c)
    N.check("mjx_vardiff_jvp2d", N.lib().mjx_vardiff_jvp2d(
        grid.nx, float(grid.dy), float(grid.dx), abc, float(a0), float(beta), N.ptr(u64), N.ptr(v64), N.ptr(out),
        N.stream_ptr(u.device)))
    return out


def _vardiff_rhs(model: MOLModel, state):
    """MOLModel.rhs of the variable-diffusion model (ghosts zeroed, as the reference ops)."""
    return _vardiff_rhs_raw(state, model.grid, model.params)


def get_fft_cache(model: MOLModel):
    return model.metadata.get("fft_cache")


def get_diffusivities(model: MOLModel) -> Dict[str, float]:
    return model.diffusivities()
