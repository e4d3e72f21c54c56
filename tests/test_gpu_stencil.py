"""Ghost cells, Laplacian and fused model RHS on the GPU vs the oracle."""

import numpy as np
import pytest
import torch

from oracle import mol

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", [mol.PERIODIC, mol.DIRICHLET, mol.NEUMANN])
def test_bc_fill_and_pad(cuda, kind):
    from moljax_gb300.core import stencil
    from moljax_gb300.core.bc import FieldBCSpec, BCType
    import moljax_gb300 as M
    g = M.Grid2D(12, 8, 0, 1.2, 0, 0.8)
    og = mol.Grid2D(12, 8, 0, 1.2, 0, 0.8)
    rng = np.random.default_rng(kind)
    f = rng.standard_normal((10, 14))
    vals = {"left": 0.3, "right": -0.2, "bottom": 0.7, "top": 1.1}
    spec = FieldBCSpec(BCType(kind), value=(lambda X, Y, t, p: vals) if kind == 1 else None,
                       flux=(lambda X, Y, t, p: vals) if kind == 2 else None)
    out = stencil.apply_bc({"u": torch.tensor(f, device=cuda)}, g, {"u": spec})["u"].cpu().numpy()
    ref = mol.bc_2d(f, og, kind, vals if kind else None)
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-15)
    pad = stencil.pad_interior(torch.tensor(f[None, 1:-1, 1:-1], device=cuda), g, {"u": spec}, ["u"])
    np.testing.assert_allclose(pad[0].cpu().numpy(), ref, rtol=0, atol=1e-15)


def test_laplacian_and_rhs(cuda):
    import moljax_gb300 as M
    from moljax_gb300.core import stencil
    g = M.Grid2D(32, 16, 0, 2.5, 0, 1.25)
    og = mol.Grid2D(32, 16, 0, 2.5, 0, 1.25)
    model = M.create_gray_scott_model(g, 2e-3, 1e-3, 0.035, 0.065)
    y = mol.gray_scott_ic(og, 9)
    lap = stencil.laplacian_2d(torch.tensor(y["u"], device=cuda), g).cpu().numpy()
    np.testing.assert_allclose(lap, mol.laplacian_2d(y["u"], og), rtol=1e-13, atol=1e-10)
    r = model.rhs({k: torch.tensor(v, device=cuda) for k, v in y.items()}, 0.0)
    yb = mol.apply_bc(y, og, {"u": 0, "v": 0})
    R = mol.gray_scott_reaction(yb, 0.035, 0.065)
    for k, D in (("u", 2e-3), ("v", 1e-3)):
        ref = D * mol.laplacian_2d(yb[k], og) + R[k]
        np.testing.assert_allclose(mol.interior(r[k].cpu().numpy(), og), mol.interior(ref, og),
                                   rtol=1e-12, atol=1e-13)
