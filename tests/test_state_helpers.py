"""StateDict helpers on CPU tensors (moljax/core/state.py, utils.py): pure tensor
plumbing, checked against direct formulas."""

import math

import torch

import moljax_gb300 as M
from moljax_gb300.core import utils as U


def test_tree_helpers_and_flatten():
    g = M.Grid2D(4, 3, 0.0, 1.0, 0.0, 1.0)
    a = {"u": torch.arange(30, dtype=torch.float64).reshape(5, 6), "v": torch.ones(5, 6, dtype=torch.float64)}
    b = {"u": torch.full((5, 6), 2.0, dtype=torch.float64), "v": torch.full((5, 6), 3.0, dtype=torch.float64)}
    assert torch.equal(M.tree_add(a, b)["u"], a["u"] + 2)
    assert torch.equal(M.tree_sub(a, b)["v"], torch.full((5, 6), -2.0, dtype=torch.float64))
    assert torch.equal(M.tree_axpy(a, 0.5, b)["u"], a["u"] + 1)
    assert torch.equal(M.tree_scale(a, 2.0)["v"], torch.full((5, 6), 2.0, dtype=torch.float64))
    ui = a["u"][1:-1, 1:-1]
    n2 = math.sqrt(float((ui ** 2).sum()) + 12.0)
    assert abs(float(M.tree_norm2(a, g)) - n2) < 1e-12
    assert float(M.tree_norm_inf(a, g)) == float(ui.max())
    assert abs(float(M.tree_vdot(a, b, g)) - (2 * float(ui.sum()) + 3 * 12)) < 1e-9
    flat, unravel = M.flatten_to_vec(a)
    assert flat.shape == (60,) and torch.equal(unravel(flat)["u"], a["u"])
    assert torch.equal(M.unflatten_from_vec(flat, a)["v"], a["v"])
    assert M.state_total_size(a) == 60 and M.state_interior_size(a, g) == 24
    st = M.create_state_from_interior({"w": torch.ones(3, 4)}, g)
    assert st["w"].shape == (5, 6) and float(st["w"].sum()) == 12.0 and float(st["w"][0].sum()) == 0.0
    assert torch.equal(M.get_interior_state(a, g)["u"], ui)


def test_utils_helpers():
    g1 = M.Grid1D(8, 0.0, 1.0)
    p = U.create_padded_array(g1, 1.5)
    assert p.shape == (10,) and float(p.sum()) == 15.0
    q = U.set_interior(p, torch.zeros(8, dtype=torch.float64), g1)
    assert float(q.sum()) == 3.0 and float(p.sum()) == 15.0
    assert float(U.sum_interior(q, g1)) == 0.0 and float(U.max_abs_interior(p, g1)) == 1.5
    h = U.allocate_state_history({"u": p}, g1, 4)
    U.save_to_history(h, {"u": p}, g1, 2)
    assert h["u"].shape == (4, 8) and float(h["u"][2].sum()) == 12.0
    assert U.eps_for_dtype(torch.float32) == 1e-10 and U.eps_for_dtype(torch.float64) == 1e-14
    st = {"u": torch.full((10, 10), 0.5), "v": torch.full((10, 10), 0.25)}
    s = M.estimate_reaction_stiffness(st, {"F": 0.035, "k": 0.065})
    assert abs(s - max(0.1, 0.25 ** 2 + 0.035, 2 * 0.5 * 0.25 + 0.1)) < 1e-12
    assert M.estimate_reaction_stiffness({}, {"r": 3.0}) == 3.0


def test_preconditioner_factories():
    pc = M.create_gray_scott_preconditioner()
    assert isinstance(pc, M.BlockJacobiPreconditioner) and pc.diffusion_keys == {"u": "Du", "v": "Dv"}
    pa = M.create_advdiff_preconditioner(["a", "b"])
    assert pa.diffusion_keys == {"a": "D", "b": "D"} and pa.advection_keys == {"a": "vx", "b": "vx"}
    pf = M.create_gray_scott_fft_preconditioner(None)
    assert pf.field_diffusivity_keys == {"u": "Du", "v": "Dv"}
    assert isinstance(M.create_diffusion_preconditioner({"u": "D"}, 3), M.DiffusionPreconditioner)
