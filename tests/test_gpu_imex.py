"""IMEX-Strang step and the adaptive device loop vs the NumPy FP64 oracle."""

import numpy as np
import pytest
import torch

from oracle import imex as OI
from oracle import mol

pytestmark = pytest.mark.gpu


def _setup(n, dtype, cuda, seed=11):
    import moljax_gb300 as M
    grid = M.Grid2D(n, n, 0.0, 2.5, 0.0, 2.5)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, dtype, cuda)
    og = mol.Grid2D(n, n, 0, 2.5, 0, 2.5)
    y0 = mol.gray_scott_ic(og, seed)
    ym = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
    omodel, lam, odiff = OI.gray_scott_periodic(og, 2e-5, 1e-5, 0.035, 0.065)
    return M, grid, model, cache, diff, ym, og, y0, omodel, lam, odiff


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("n", [16, 64, 256, 1024])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_strang_step_vs_oracle(cuda, n, dtype):
    """One IMEX-Strang step; at 1024 the FP32 row passes take the one-warp-per-row form."""
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(n, dtype, cuda)
    out = M.imex_strang_step(model, ym, 0.0, 0.8, cache, diff)
    ref = OI.imex_strang_step(om, y0, 0.8, lam, od)
    tol = 1e-13 if dtype == torch.float64 else 2e-6
    for k in ("u", "v"):
        assert _rel(out[k].cpu().numpy(), ref[k]) < tol  # ghosts included (periodic fill)


def test_adaptive_fp64_matches_oracle_counts(cuda):
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(32, torch.float64, cuda)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 40.0, 1.0, cache, diff, pid_params=pid,
                                  save_every=1, max_steps=2000)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 40.0, 1.0, lam, od,
                                    pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=1,
                                    max_steps=2000)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    assert r.t_final == pytest.approx(ro.t_final, abs=1e-12)
    for k in ("u", "v"):
        assert _rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-11
    nh = ro.n_steps
    assert r.n_steps == nh
    # dt comes from err_ratio, a norm of y_half2 - y_full (cancellation): ~1e-11 relative noise
    np.testing.assert_allclose(r.t_history.cpu().numpy()[:nh], ro.t_history[:nh], rtol=1e-9)
    np.testing.assert_allclose(r.dt_history.cpu().numpy()[:nh], ro.dt_history[:nh], rtol=1e-9)
    for k in ("u", "v"):
        assert _rel(r.y_history[k][:nh].cpu().numpy(), ro.y_history[k][:nh]) < 1e-11


def test_adaptive_fp32_close_to_fp64_oracle(cuda):
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(64, torch.float32, cuda)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 20.0, 1.0, cache, diff, pid_params=pid,
                                  save_every=1000, save_y_history=False)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 20.0, 1.0, lam, od,
                                    pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=1000,
                                    keep_history=False)
    assert r.status == ro.status == 0
    assert abs(r.n_accepted - ro.n_accepted) <= 2
    for k in ("u", "v"):
        assert _rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-5


def test_adaptive_nonfinite_status(cuda):
    # a NaN in the initial data: the first attempt is rejected and the run stops
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(16, torch.float64, cuda)
    ym["u"][5, 5] = float("nan")
    r = M.adaptive_integrate_imex(model, ym, 0.0, 10.0, 1.0, cache, diff)
    assert r.status == M.StatusCode.NON_FINITE_VALUES
    assert r.n_accepted == 0 and r.n_rejected == 1


def test_adaptive_dt_too_small(cuda):
    # impossible tolerance with dt_min close to dt: DT_TOO_SMALL as the reference
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(16, torch.float64, cuda)
    pid = M.PIDParams(atol=1e-30, rtol=1e-30, dt_min=0.3)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 10.0, 1.0, cache, diff, pid_params=pid)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 10.0, 1.0, lam, od,
                                    pid=OI.PIDParams(atol=1e-30, rtol=1e-30, dt_min=0.3))
    assert r.status == ro.status == M.StatusCode.DT_TOO_SMALL
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)


def test_adaptive_max_steps(cuda):
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(16, torch.float64, cuda)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 100.0, 1.0, cache, diff, max_steps=5)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 100.0, 1.0, lam, od, max_steps=5)
    assert r.status == ro.status == M.StatusCode.MAX_STEPS_REACHED
    assert r.n_accepted == ro.n_accepted == 5


@pytest.mark.parametrize("n", [32, 128])
def test_adaptive_mixed_precision_vs_oracle(cuda, n):
    # FP64 spectral state + FP32 increment transforms: FP64-level accuracy, same step counts
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(n, torch.float32, cuda)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 30.0, 1.0, cache, diff, pid_params=pid,
                                  save_every=100, precision="mixed")
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 30.0, 1.0, lam, od,
                                    pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=100,
                                    keep_history=False)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    for k in ("u", "v"):
        assert _rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-6
    rf = M.adaptive_integrate_imex(model, ym, 0.0, 30.0, 1.0, cache, diff, pid_params=pid,
                                   save_every=100, save_y_history=False, precision="fp32")
    e_mixed = max(_rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) for k in ("u", "v"))
    e_fp32 = max(_rel(rf.y_final[k].cpu().numpy(), ro.y_final[k]) for k in ("u", "v"))
    assert e_mixed < e_fp32


_HOST_LOOP_CHILD = r"""
import sys, numpy as np, torch
sys.path.insert(0, sys.argv[1])
import moljax_gb300 as M
from oracle import mol
dev = torch.device("cuda", 0)
ny, nx = int(sys.argv[3]), int(sys.argv[4])
out = {}
for prec, dtype in (("fp64", torch.float64), ("fp32", torch.float32), ("mixed", torch.float32)):
    grid = M.Grid2D(nx, ny, 0.0, 2.5, 0.0, 2.5)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, dtype, dev)
    y0 = mol.gray_scott_ic(mol.Grid2D(nx, ny, 0, 2.5, 0, 2.5), 11)
    ym = {k: torch.tensor(v, dtype=dtype, device=dev) for k, v in y0.items()}
    r = M.adaptive_integrate_imex(model, ym, 0.0, 25.0, 1.0, cache, diff,
                                  pid_params=M.PIDParams(atol=1e-7, rtol=1e-5), save_every=3,
                                  max_steps=2000, precision=prec)
    out[prec + "_u"] = r.y_final["u"].cpu().numpy()
    out[prec + "_counts"] = np.array([r.n_accepted, r.n_rejected, r.status])
    out[prec + "_t"] = r.t_history.cpu().numpy()
np.savez(sys.argv[2], **out)
"""


@pytest.mark.parametrize("ny,nx", [(64, 64), (32, 1024)])
def test_host_driven_loop_matches_device_loop(cuda, tmp_path, ny, nx):
    # MJX_HOST_LOOP=1 (read once per process) launches the attempts from the host in
    # batches instead of the conditional graph: identical kernels, identical results, bit for
    # bit.  Rows of 1024 take the warp-row pass.
    import os
    import subprocess
    import sys
    from oracle import mol as omol
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    path = str(tmp_path / "child.npz")
    env = dict(os.environ, MJX_HOST_LOOP="1")
    subprocess.run([sys.executable, "-c", _HOST_LOOP_CHILD, root, path, str(ny), str(nx)], env=env,
                   check=True, timeout=600)
    child = np.load(path)
    import moljax_gb300 as M
    for prec, dtype in (("fp64", torch.float64), ("fp32", torch.float32), ("mixed", torch.float32)):
        grid = M.Grid2D(nx, ny, 0.0, 2.5, 0.0, 2.5)
        model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, dtype, cuda)
        y0 = omol.gray_scott_ic(omol.Grid2D(nx, ny, 0, 2.5, 0, 2.5), 11)
        ym = {k: torch.tensor(v, dtype=dtype, device=cuda) for k, v in y0.items()}
        r = M.adaptive_integrate_imex(model, ym, 0.0, 25.0, 1.0, cache, diff,
                                      pid_params=M.PIDParams(atol=1e-7, rtol=1e-5), save_every=3,
                                      max_steps=2000, precision=prec)
        assert list(child[prec + "_counts"]) == [r.n_accepted, r.n_rejected, r.status]
        np.testing.assert_array_equal(child[prec + "_u"], r.y_final["u"].cpu().numpy())
        np.testing.assert_array_equal(child[prec + "_t"], r.t_history.cpu().numpy())


@pytest.mark.parametrize("n", [16, 128])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_imex_euler_step_vs_oracle(cuda, n, dtype):
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(n, dtype, cuda)
    out = M.imex_euler_step(model, ym, 0.0, 0.8, cache, diff)
    ref = OI.imex_euler_step(om, y0, 0.8, lam, od)
    tol = 1e-13 if dtype == torch.float64 else 2e-6
    for k in ("u", "v"):
        assert _rel(out[k].cpu().numpy(), ref[k]) < tol


def test_imex_euler_fixed_dt_vs_oracle(cuda):
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(32, torch.float64, cuda)
    t, ys, yf = M.integrate_imex_fixed_dt(model, ym, 0.0, 4.0, 0.5, cache, diff, use_strang=False)
    to, yo, yfo = OI.integrate_imex_fixed_dt(om, y0, 0.0, 4.0, 0.5, lam, od, use_strang=False)
    np.testing.assert_allclose(t.numpy(), np.asarray(to), rtol=1e-14)
    for k in ("u", "v"):
        assert _rel(yf[k].cpu().numpy(), yfo[k]) < 1e-12


def test_adaptive_imex_euler_matches_oracle_counts(cuda):
    # order-1 step doubling: same accept/reject sequence and result as the oracle
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(32, torch.float64, cuda)
    pid = M.PIDParams(atol=1e-6, rtol=1e-4)
    r = M.adaptive_integrate(model, ym, 0.0, 15.0, 1.0, M.IntegratorType.IMEX_EULER,
                             max_steps=5000, pid_params=pid, save_every=1)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 15.0, 1.0, lam, od, use_strang=False,
                                    pid=OI.PIDParams(atol=1e-6, rtol=1e-4), save_every=1,
                                    max_steps=5000)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    assert r.n_rejected > 0 or r.n_accepted > 5
    nh = ro.n_steps
    np.testing.assert_allclose(r.t_history.cpu().numpy()[:nh], ro.t_history[:nh], rtol=1e-9)
    for k in ("u", "v"):
        assert _rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-10


def test_adaptive_imex_euler_fp32(cuda):
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(64, torch.float32, cuda)
    pid = M.PIDParams(atol=1e-6, rtol=1e-4)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 10.0, 1.0, cache, diff, use_strang=False,
                                  pid_params=pid, save_every=1000, save_y_history=False)
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 10.0, 1.0, lam, od, use_strang=False,
                                    pid=OI.PIDParams(atol=1e-6, rtol=1e-4), save_every=1000,
                                    keep_history=False)
    assert r.status == ro.status == 0
    assert abs(r.n_accepted - ro.n_accepted) <= 2
    for k in ("u", "v"):
        assert _rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-5


def test_history_streamed_to_host_equals_device_history(cuda):
    # save_y_history="host": the history kernel writes pinned host memory directly
    M, grid, model, cache, diff, ym, og, y0, om, lam, od = _setup(64, torch.float32, cuda)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    kw = dict(pid_params=pid, save_every=2, max_steps=400, precision="fp32")
    rd = M.adaptive_integrate_imex(model, ym, 0.0, 12.0, 1.0, cache, diff, save_y_history=True, **kw)
    rh = M.adaptive_integrate_imex(model, ym, 0.0, 12.0, 1.0, cache, diff, save_y_history="host", **kw)
    assert rh.y_history["u"].device.type == "cpu" and rh.y_history["u"].is_pinned()
    assert (rd.n_accepted, rd.n_steps) == (rh.n_accepted, rh.n_steps)
    k = rd.n_steps
    for f in ("u", "v"):
        np.testing.assert_array_equal(rh.y_history[f][:k].numpy(), rd.y_history[f][:k].cpu().numpy())


@pytest.mark.parametrize("ny,nx", [(4096, 32), (32, 4096)])
def test_adaptive_mixed_maximum_extent(cuda, ny, nx):
    # the largest transform length (4096) along each axis: one-column 512-thread column
    # tiles (ny = 4096) and 4096-point row transforms (nx = 4096)
    import moljax_gb300 as M
    L = 2.5
    grid = M.Grid2D(nx, ny, 0.0, L, 0.0, L)
    model, cache, diff = M.create_gray_scott_periodic_fft(grid, 2e-5, 1e-5, 0.035, 0.065, torch.float32, cuda)
    og = mol.Grid2D(nx, ny, 0, L, 0, L)
    y0 = mol.gray_scott_ic(og, 17)
    ym = {k: torch.tensor(v, dtype=torch.float32, device=cuda) for k, v in y0.items()}
    om, lam, od = OI.gray_scott_periodic(og, 2e-5, 1e-5, 0.035, 0.065)
    pid = M.PIDParams(atol=1e-7, rtol=1e-5)
    r = M.adaptive_integrate_imex(model, ym, 0.0, 12.0, 1.0, cache, diff, pid_params=pid,
                                  save_every=100, save_y_history=False, precision="mixed")
    ro = OI.adaptive_integrate_imex(om, y0, 0.0, 12.0, 1.0, lam, od,
                                    pid=OI.PIDParams(atol=1e-7, rtol=1e-5), save_every=100,
                                    keep_history=False)
    assert r.status == ro.status == 0
    assert (r.n_accepted, r.n_rejected) == (ro.n_accepted, ro.n_rejected)
    for k in ("u", "v"):
        assert _rel(r.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-6
    rf = M.adaptive_integrate_imex(model, ym, 0.0, 12.0, 1.0, cache, diff, pid_params=pid,
                                   save_every=100, save_y_history=False, precision="fp32")
    assert rf.status == 0
    for k in ("u", "v"):
        assert _rel(rf.y_final[k].cpu().numpy(), ro.y_final[k]) < 1e-4
