"""Explicit Runge-Kutta steppers (fused stencil stages) vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import explicit as OX
from oracle import imex as OI
from oracle import mol

pytestmark = pytest.mark.gpu

SIDES = {"left": 0.2, "right": -0.1, "bottom": 0.05, "top": 0.3}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _gs(n, kind, cuda, dtype=torch.float64):
    import moljax_gb300 as M
    from moljax_gb300.core.bc import FieldBCSpec, BCType
    grid = M.Grid2D(n, n, 0.0, 2.5, 0.0, 2.5)
    model = M.create_gray_scott_model(grid, 2e-5, 1e-5, 0.035, 0.065, BCType(kind), dtype)
    vals = None
    if kind != mol.PERIODIC:
        fn = (lambda X, Y, t, p: dict(SIDES))
        spec = FieldBCSpec(kind=BCType(kind), value=fn) if kind == mol.DIRICHLET else \
            FieldBCSpec(kind=BCType(kind), flux=fn)
        model = M.MOLModel(model.grid, {"u": spec, "v": spec}, model.params, model.linear_ops,
                           model.nonlinear_ops, model.metadata)
        vals = {"u": dict(SIDES), "v": dict(SIDES)}
    og = mol.Grid2D(n, n, 0, 2.5, 0, 2.5)
    y0 = mol.gray_scott_ic(og, 5)
    om = OX.ExplicitModel(og, {"u": kind, "v": kind}, {"u": 2e-5, "v": 1e-5}, vals or {},
                          lambda y: mol.gray_scott_reaction(y, 0.035, 0.065),
                          params={"Du": 2e-5, "Dv": 1e-5, "F": 0.035, "k": 0.065})
    ym = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
    return M, model, ym, om, y0


def _advdiff(n, kind, upwind, cuda, vx=1.0, vy=-0.5):
    import moljax_gb300 as M
    from moljax_gb300.core.bc import BCType
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_advection_diffusion_model(grid, ["c1", "c2"], 0.01, vx, vy, BCType(kind), upwind)
    og = mol.Grid2D(n, n, 0, 1, 0, 1)
    rng = np.random.default_rng(3)
    y0 = {k: mol.pad(rng.uniform(0, 1, (n, n)), og) for k in ("c1", "c2")}
    om = OX.ExplicitModel(og, {"c1": kind, "c2": kind}, {"c1": 0.01, "c2": 0.01},
                          advection="upwind" if upwind else "central", vx=vx, vy=vy,
                          params={"D": 0.01, "vx": vx, "vy": vy})
    ym = {k: torch.tensor(v, device=cuda) for k, v in y0.items()}
    return M, model, ym, om, y0


def _interior(a, n):
    return a[1:n + 1, 1:n + 1]


@pytest.mark.parametrize("kind", [mol.PERIODIC, mol.DIRICHLET, mol.NEUMANN])
def test_rhs_vs_oracle(cuda, kind):
    n = 32
    M, model, ym, om, y0 = _gs(n, kind, cuda)
    F = model.rhs(ym)
    R = om.rhs(y0)
    for k in ("u", "v"):
        assert _rel(_interior(F[k].cpu().numpy(), n), _interior(R[k], n)) < 1e-12
    for upwind in (True, False):
        M, model, ym, om, y0 = _advdiff(n, kind, upwind, cuda)
        F = model.rhs(ym)
        R = om.rhs(y0)
        for k in ("c1", "c2"):
            assert _rel(_interior(F[k].cpu().numpy(), n), _interior(R[k], n)) < 1e-12


@pytest.mark.parametrize("method", [0, 1, 2])
@pytest.mark.parametrize("kind", [mol.PERIODIC, mol.DIRICHLET, mol.NEUMANN])
def test_single_steps_vs_oracle(cuda, method, kind):
    n = 32
    step = {0: "euler_step", 1: "ssprk3_step", 2: "rk4_step"}[method]
    M, model, ym, om, y0 = _gs(n, kind, cuda)
    out = getattr(M, step)(model, ym, 0.0, 0.7)
    ref = OX.STEPS[method](om, y0, 0.7)
    for k in ("u", "v"):
        assert _rel(_interior(out[k].cpu().numpy(), n), _interior(ref[k], n)) < 1e-13
    M, model, ym, om, y0 = _advdiff(n, kind, True, cuda)
    out = getattr(M, step)(model, ym, 0.0, 2e-3)
    ref = OX.STEPS[method](om, y0, 2e-3)
    for k in ("c1", "c2"):
        assert _rel(_interior(out[k].cpu().numpy(), n), _interior(ref[k], n)) < 1e-13


def test_integrate_fixed_dt_rk4(cuda):
    n = 32
    M, model, ym, om, y0 = _advdiff(n, mol.PERIODIC, True, cuda)
    t, ys, yf = M.integrate_fixed_dt(model, ym, 0.0, 0.02, 4e-3, M.IntegratorType.RK4)
    assert t.numel() == 6 and ys["c1"].shape[0] == 6
    y = y0
    for _ in range(6):
        y = OX.rk4_step(om, y, 4e-3)
    for k in ("c1", "c2"):
        assert _rel(_interior(yf[k].cpu().numpy(), n), _interior(y[k], n)) < 1e-12


@pytest.mark.parametrize("method", [0, 1, 2])
def test_adaptive_explicit_vs_oracle(cuda, method):
    # step doubling + PI + CFL limit: same accept/reject sequence as the oracle
    n = 32
    M, model, ym, om, y0 = _gs(n, mol.NEUMANN, cuda)
    itype = [M.IntegratorType.EULER, M.IntegratorType.SSPRK3, M.IntegratorType.RK4][method]
    pid = M.PIDParams(atol=1e-6, rtol=1e-4)
    r = M.adaptive_integrate(model, ym, 0.0, 30.0, 1.0, itype, max_steps=4000, pid_params=pid,
                             save_every=1)
    ro = OX.adaptive_integrate_explicit(om, y0, 0.0, 30.0, 1.0, method, max_steps=4000,
                                        pid=OI.PIDParams(atol=1e-6, rtol=1e-4), save_every=1)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    k = ro.n_steps
    np.testing.assert_allclose(r.t_history.cpu().numpy()[:k], ro.t_history[:k], rtol=1e-9)
    for f in ("u", "v"):
        assert _rel(_interior(r.y_final[f].cpu().numpy(), n), _interior(ro.y_final[f], n)) < 1e-10
    assert r.y_history["u"].shape[0] == 4001


def test_adaptive_advection_cfl_limited(cuda):
    # advection-diffusion: dt is capped by heisenberg_cfl_dt (0.9 * 0.5 dx / |v|)
    n = 32
    M, model, ym, om, y0 = _advdiff(n, mol.PERIODIC, True, cuda)
    pid = M.PIDParams(atol=1e-3, rtol=1e-2)
    r = M.adaptive_integrate(model, ym, 0.0, 0.2, 1.0, M.IntegratorType.SSPRK3, max_steps=4000,
                             pid_params=pid, save_every=1, save_y_history=False)
    ro = OX.adaptive_integrate_explicit(om, y0, 0.0, 0.2, 1.0, 1, max_steps=4000,
                                        pid=OI.PIDParams(atol=1e-3, rtol=1e-2), save_every=1)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    dt_cfl = 0.9 * 0.5 * (1 / n) / 1.5
    assert float(r.dt_history[: r.n_steps - 1].max()) <= dt_cfl * (1 + 1e-12)
    for f in ("c1", "c2"):
        assert _rel(_interior(r.y_final[f].cpu().numpy(), n), _interior(ro.y_final[f], n)) < 1e-10


def test_fft_preconditioners_vs_oracle(cuda):
    import moljax_gb300 as M
    n = 64
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.5)
    cache = M.create_fft_cache(grid, torch.float64, cuda)
    og = mol.Grid2D(n, n, 0, 1, 0, 1.5)
    rng = np.random.default_rng(9)
    r = rng.standard_normal((n, n))
    params = {"D": 0.02, "v": (1.3, -0.7), "vs": 0.4}
    ctx = M.PrecondContext(grid, 0.05, params)
    P = M.FFTAdvectionDiffusionPreconditioner(field_diffusivity_keys={"a": "D", "b": "D"},
                                              field_velocity_keys={"a": "v", "b": "vs"},
                                              fft_cache=cache)
    padded = torch.zeros((n + 2, n + 2), dtype=torch.float64, device=cuda)
    padded[1:-1, 1:-1] = torch.tensor(r, device=cuda)
    padded[0, :] = 7.0
    out = P.apply({"a": torch.tensor(r, device=cuda), "b": padded}, ctx)
    ref_a = OX.fft_advdiff_inverse(r, og, 0.05, 0.02, 1.3, -0.7)
    ref_b = OX.fft_advdiff_inverse(r, og, 0.05, 0.02, 0.4, 0.0)
    assert _rel(out["a"].cpu().numpy(), ref_a) < 1e-12
    assert _rel(out["b"][1:-1, 1:-1].cpu().numpy(), ref_b) < 1e-12
    assert float(out["b"][0, 3]) == 7.0  # ghosts kept
    Q = M.FFTDiffusionPreconditioner(field_diffusivity_keys={"a": "D"}, fft_cache=cache)
    q = Q.apply({"a": torch.tensor(r, device=cuda)}, ctx)["a"].cpu().numpy()
    assert _rel(q, OX.fft_advdiff_inverse(r, og, 0.05, 0.02, 0.0, 0.0)) < 1e-12


def test_2d_derivatives_error_norm_is_finite(cuda):
    import moljax_gb300 as M
    n = 24
    grid = M.Grid2D(n, n + 8, 0.0, 1.0, 0.0, 2.0)
    og = mol.Grid2D(n, n + 8, 0, 1, 0, 2)
    rng = np.random.default_rng(4)
    f = rng.standard_normal((n + 10, n + 2))  # ghosts included, read as stored
    ft = torch.tensor(f, device=cuda)
    for axis in (0, 1):
        for v in (0.7, -0.3):
            got = M.d1_upwind_2d(ft, v, grid, axis).cpu().numpy()
            np.testing.assert_allclose(got, mol.d1_upwind_2d(f, v, og, axis), rtol=1e-13, atol=1e-13)
    got = M.d1_central_2d(ft, grid, 1).cpu().numpy()
    np.testing.assert_allclose(got, OX._central(f, og, 1), rtol=1e-13, atol=1e-13)
    e = {"u": torch.tensor(rng.standard_normal(f.shape), device=cuda), "v": ft * 1e-3}
    y = {"u": ft, "v": ft + 2.0}
    ref = mol.scaled_error_norm({k: t.cpu().numpy() for k, t in e.items()},
                                {k: t.cpu().numpy() for k, t in y.items()}, og, 1e-6, 1e-4)
    assert M.scaled_error_norm(e, y, grid, 1e-6, 1e-4) == pytest.approx(ref, rel=1e-12)
    assert M.is_finite(y)
    y["v"] = y["v"].clone()
    y["v"][3, 4] = float("nan")
    assert not M.is_finite(y)


@pytest.mark.parametrize("shape", [(70, 33), (5, 1), (3, 65), (97, 129), (130, 64), (40, 70), (12, 36)])
@pytest.mark.parametrize("kind", [mol.PERIODIC, mol.DIRICHLET, mol.NEUMANN])
def test_stage_tiles_any_shape(cuda, shape, kind):
    """The stage kernel's 32 x 64 tiles on grids that leave partial tiles, a one-column last
    tile (nx = 33, 65, 129) and single-column grids; three fields (the four-field build),
    SSPRK3 and RK4, BC values on every side."""
    import moljax_gb300 as M
    from moljax_gb300.core.bc import FieldBCSpec, BCType
    ny, nx = shape
    names = ("c1", "c2", "c3")
    grid = M.Grid2D(nx, ny, 0.0, 1.0, 0.0, 0.8)
    og = mol.Grid2D(nx, ny, 0, 1, 0, 0.8)
    model = M.create_advection_diffusion_model(grid, names, 0.01, 0.7, -0.4, BCType(kind), True)
    vals = {}
    if kind != mol.PERIODIC:
        fn = (lambda X, Y, t, p: dict(SIDES))
        spec = FieldBCSpec(kind=BCType(kind), value=fn) if kind == mol.DIRICHLET else \
            FieldBCSpec(kind=BCType(kind), flux=fn)
        model = M.MOLModel(model.grid, {k: spec for k in names}, model.params, model.linear_ops,
                           model.nonlinear_ops, model.metadata)
        vals = {k: dict(SIDES) for k in names}
    om = OX.ExplicitModel(og, {k: kind for k in names}, {k: 0.01 for k in names}, vals,
                          advection="upwind", vx=0.7, vy=-0.4, params={"D": 0.01, "vx": 0.7, "vy": -0.4})
    rng = np.random.default_rng(ny * 131 + nx)
    y0 = {k: mol.pad(rng.uniform(0, 1, (ny, nx)), og) for k in names}
    ym = {k: torch.tensor(v, device=cuda) for k, v in y0.items()}
    c = (slice(1, ny + 1), slice(1, nx + 1))
    for method, step in ((1, "ssprk3_step"), (2, "rk4_step")):
        out = getattr(M, step)(model, ym, 0.0, 1e-3)
        ref = OX.STEPS[method](om, y0, 1e-3)
        for k in names:
            np.testing.assert_allclose(out[k].cpu().numpy()[c], ref[k][c], rtol=0, atol=1e-12)
    # FP32 state: the same RK4 step within single-precision rounding
    m32 = M.create_advection_diffusion_model(grid, names, 0.01, 0.7, -0.4, BCType(kind), True,
                                             dtype=torch.float32)
    if kind != mol.PERIODIC:
        m32 = M.MOLModel(m32.grid, model.bc_spec, m32.params, m32.linear_ops, m32.nonlinear_ops, m32.metadata)
    out = M.rk4_step(m32, {k: v.float() for k, v in ym.items()}, 0.0, 1e-3)
    ref = OX.STEPS[2](om, y0, 1e-3)
    for k in names:
        np.testing.assert_allclose(out[k].cpu().double().numpy()[c], ref[k][c], rtol=0, atol=2e-5)


def test_gray_scott_stage_rectangular(cuda):
    """Gray-Scott (the two-field reaction build) on a 48 x 80 grid with Dirichlet values."""
    import moljax_gb300 as M
    from moljax_gb300.core.bc import FieldBCSpec, BCType
    ny, nx = 48, 80
    grid = M.Grid2D(nx, ny, 0.0, 2.5, 0.0, 1.5)
    model = M.create_gray_scott_model(grid, 2e-5, 1e-5, 0.035, 0.065, BCType(mol.DIRICHLET))
    fn = (lambda X, Y, t, p: dict(SIDES))
    spec = FieldBCSpec(kind=BCType(mol.DIRICHLET), value=fn)
    model = M.MOLModel(model.grid, {"u": spec, "v": spec}, model.params, model.linear_ops,
                       model.nonlinear_ops, model.metadata)
    og = mol.Grid2D(nx, ny, 0, 2.5, 0, 1.5)
    y0 = mol.gray_scott_ic(og, 9)
    om = OX.ExplicitModel(og, {"u": mol.DIRICHLET, "v": mol.DIRICHLET}, {"u": 2e-5, "v": 1e-5},
                          {"u": dict(SIDES), "v": dict(SIDES)}, lambda y: mol.gray_scott_reaction(y, 0.035, 0.065),
                          params={"Du": 2e-5, "Dv": 1e-5, "F": 0.035, "k": 0.065})
    ym = {k: torch.tensor(v, device=cuda) for k, v in y0.items()}
    c = (slice(1, ny + 1), slice(1, nx + 1))
    out = M.rk4_step(model, ym, 0.0, 0.5)
    ref = OX.STEPS[2](om, y0, 0.5)
    for k in ("u", "v"):
        np.testing.assert_allclose(out[k].cpu().numpy()[c], ref[k][c], rtol=0, atol=1e-13)


def _kinetics_case(n, nspecies, kind, cuda, dtype=torch.float64):
    """A mass-action network on an advection-diffusion model (the multispecies caller of
    make_reaction_op, examples/advdiff_multispecies.py, with native reactions)."""
    import moljax_gb300 as M
    from moljax_gb300.core.bc import BCType
    names = ["a", "b", "c", "d"][:nspecies]
    reactions = [(2.0, {"a": 1, "b": 1}, {"c": 1}) if nspecies >= 3 else (2.0, {"a": 1, "b": 1}, {}),
                 (0.7, {"b": 2}, {"a": 1}), (0.25, {"a": 1}, {"a": 2}), (0.1, {"a": 3}, {})]
    if nspecies == 4:
        reactions.append((1.3, {"c": 1, "d": 1}, {"d": 2}))
    linear = {("a", "b"): 0.3, ("b", "b"): -0.3}
    source = {"b": 0.05}
    op = M.make_kinetics_op(names, reactions, linear, source)
    grid = M.Grid2D(n, n, 0.0, 1.0, 0.0, 1.0)
    model = M.create_advection_diffusion_model(grid, names, 0.01, 0.6, -0.4, BCType(kind), True, dtype,
                                               reactions=op)
    og = mol.Grid2D(n, n, 0, 1, 0, 1)
    rng = np.random.default_rng(17)
    y0 = {k: mol.pad(rng.uniform(0.2, 1.0, (n, n)), og) for k in names}
    om = OX.ExplicitModel(og, {k: kind for k in names}, {k: 0.01 for k in names}, advection="upwind",
                          vx=0.6, vy=-0.4, reaction=OX.mass_action(names, reactions, linear, source),
                          params={"D": 0.01, "vx": 0.6, "vy": -0.4})
    ym = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
    return M, model, ym, om, y0, names


@pytest.mark.parametrize("nspecies", [2, 3, 4])
@pytest.mark.parametrize("kind", [mol.PERIODIC, mol.NEUMANN])
def test_kinetics_network_vs_oracle(cuda, nspecies, kind):
    """The native mass-action network in the RHS, in SSPRK3 / RK4 steps (scalar and 128-bit
    stage kernels: n = 32 and 34 columns) and in the adaptive loop, against the oracle."""
    for n in (32, 34):
        M, model, ym, om, y0, names = _kinetics_case(n, nspecies, kind, cuda)
        F = model.rhs(ym)
        R = om.rhs(y0)
        for k in names:
            assert _rel(_interior(F[k].cpu().numpy(), n), _interior(R[k], n)) < 1e-12
        # the torch form of the op (generic paths) gives the same rates
        Rt = model.nonlinear_ops[0].apply(ym, model.grid, 0.0, model.params)
        Ro = om.reaction(y0)
        for k in names:
            assert _rel(_interior(Rt[k].cpu().numpy(), n), _interior(Ro[k], n)) < 1e-13
        for method in (1, 2):
            step = {1: "ssprk3_step", 2: "rk4_step"}[method]
            out = getattr(M, step)(model, ym, 0.0, 5e-3)
            ref = OX.STEPS[method](om, y0, 5e-3)
            for k in names:
                assert _rel(_interior(out[k].cpu().numpy(), n), _interior(ref[k], n)) < 1e-13
    pid = M.PIDParams(atol=1e-6, rtol=1e-4)
    r = M.adaptive_integrate(model, ym, 0.0, 0.3, 0.01, M.IntegratorType.RK4, max_steps=2000, pid_params=pid,
                             save_every=1)
    ro = OX.adaptive_integrate_explicit(om, y0, 0.0, 0.3, 0.01, 2, max_steps=2000,
                                        pid=OI.PIDParams(atol=1e-6, rtol=1e-4), save_every=1)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    for k in names:
        assert _rel(_interior(r.y_final[k].cpu().numpy(), n), _interior(ro.y_final[k], n)) < 1e-10


@pytest.mark.parametrize("shape", [(70, 300), (33, 132), (5, 4), (1, 8), (64, 256)])
@pytest.mark.parametrize("kind", [mol.PERIODIC, mol.DIRICHLET, mol.NEUMANN])
def test_tma_stage_form(cuda, shape, kind):
    """The TMA-staged stage kernel (FP32, rows a multiple of 4 points; selected by
    installing 64 as the tile height): partial tiles in x and y, grids narrower than one
    box, a single row; three fields (the four-field build) and Gray-Scott (the two-field
    reaction build); BC values on every side.  Its RHS equals the 128-bit register form bit
    for bit and the oracle within FP32 rounding; the adaptive RK4 loop (the error fused into
    the last stage) takes the same accept/reject sequence to the same state within FP32
    rounding (the error partials are summed in another order, so dt may differ in the last
    bit)."""
    import moljax_gb300 as M
    from moljax_gb300.core import autotune as AT
    from moljax_gb300.core.bc import FieldBCSpec, BCType
    ny, nx = shape
    names = ("c1", "c2", "c3")
    grid = M.Grid2D(nx, ny, 0.0, 1.0, 0.0, 0.8)
    og = mol.Grid2D(nx, ny, 0, 1, 0, 0.8)
    model = M.create_advection_diffusion_model(grid, names, 0.01, 0.7, -0.4, BCType(kind), True,
                                               dtype=torch.float32)
    vals = {}
    if kind != mol.PERIODIC:
        fn = (lambda X, Y, t, p: dict(SIDES))
        spec = FieldBCSpec(kind=BCType(kind), value=fn) if kind == mol.DIRICHLET else \
            FieldBCSpec(kind=BCType(kind), flux=fn)
        model = M.MOLModel(model.grid, {k: spec for k in names}, model.params, model.linear_ops,
                           model.nonlinear_ops, model.metadata)
        vals = {k: dict(SIDES) for k in names}
    om = OX.ExplicitModel(og, {k: kind for k in names}, {k: 0.01 for k in names}, vals,
                          advection="upwind", vx=0.7, vy=-0.4, params={"D": 0.01, "vx": 0.7, "vy": -0.4})
    rng = np.random.default_rng(ny * 7 + nx)
    y0 = {k: mol.pad(rng.uniform(0, 1, (ny, nx)), og) for k in names}
    ym = {k: torch.tensor(v, dtype=torch.float32, device=cuda) for k, v in y0.items()}
    c = (slice(1, ny + 1), slice(1, nx + 1))
    gs_grid = M.Grid2D(nx, ny, 0.0, 2.5, 0.0, 2.0)
    gs = M.create_gray_scott_model(gs_grid, 2e-5, 1e-5, 0.035, 0.065, BCType(kind), torch.float32)
    if kind != mol.PERIODIC:
        gs = M.MOLModel(gs.grid, {k: model.bc_spec["c1"] for k in ("u", "v")}, gs.params, gs.linear_ops,
                        gs.nonlinear_ops, gs.metadata)
    yg = {k: torch.tensor(v, dtype=torch.float32, device=cuda)
          for k, v in mol.gray_scott_ic(mol.Grid2D(nx, ny, 0, 2.5, 0, 2.0), 4).items()}
    pid = M.PIDParams(atol=1e-5, rtol=1e-3)
    runs = {}
    try:
        for rows in (64, 8):
            AT.set_stencil_rows(ny, nx, 3, torch.float32, rows)
            AT.set_stencil_rows(ny, nx, 2, torch.float32, rows)
            out = {"rhs": model.rhs(ym), "gs": gs.rhs(yg)}
            r = M.adaptive_integrate(model, ym, 0.0, 0.02, 1e-3, M.IntegratorType.RK4, max_steps=500,
                                     pid_params=pid, save_every=1)
            out["adaptive"] = (r.status, r.n_accepted, r.n_rejected, r.y_final)
            runs[rows] = out
    finally:
        AT.set_stencil_rows(ny, nx, 3, torch.float32, 0)
        AT.set_stencil_rows(ny, nx, 2, torch.float32, 0)
    t, v = runs[64], runs[8]
    for key in ("rhs", "gs"):
        for k in t[key]:
            assert torch.equal(t[key][k], v[key][k]), (key, k)
    assert t["adaptive"][:3] == v["adaptive"][:3] and t["adaptive"][0] == 0
    for k in names:
        torch.testing.assert_close(t["adaptive"][3][k], v["adaptive"][3][k], rtol=1e-5, atol=1e-6)
    R = om.rhs(y0)
    for k in names:
        F = t["rhs"][k].cpu().double().numpy()[c]
        assert _rel(F, R[k][c]) < 2e-5, k
