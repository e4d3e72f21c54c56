"""Seeded synthetic workloads (initial data for the benchmark configurations).

``gray_scott_initial_condition`` restates the Gray-Scott initial condition of
examples/gray_scott_2d.py:42-73: u = 1, v = 0 except the central square
|x-cx| < 0.1 Lx, |y-cy| < 0.1 Ly where u = 0.5, v = 0.25, plus 0.01*U[-1,1]
noise on the padded arrays.  The reference draws the noise from
jax.random.PRNGKey(42); here it comes from numpy.random.default_rng(seed).

``gray_scott_benchmark_ic`` is the initial condition of the reference's Gray-Scott
method benchmark (benchmarks/benchmark_gray_scott.py:59-68), drawn from numpy's
legacy seed-42 stream exactly as the script does.
"""

from __future__ import annotations

import numpy as np
import torch


def gray_scott_initial_condition(grid, seed: int = 20261203, dtype=torch.float32, device="cuda",
                                 noise: float = 0.01, frac: float = 0.1):
    X, Y = (t.numpy() for t in grid.meshgrid(include_ghost=True))
    cx = 0.5 * (grid.x_min + grid.x_max)
    cy = 0.5 * (grid.y_min + grid.y_max)
    Lx = grid.x_max - grid.x_min
    Ly = grid.y_max - grid.y_min
    mask = (np.abs(X - cx) < frac * Lx) & (np.abs(Y - cy) < frac * Ly)
    u = np.where(mask, 0.5, 1.0)
    v = np.where(mask, 0.25, 0.0)
    rng = np.random.default_rng(seed)
    u = u + noise * rng.uniform(-1.0, 1.0, u.shape)
    v = v + noise * rng.uniform(-1.0, 1.0, v.shape)
    return {"u": torch.tensor(u, dtype=dtype, device=device),
            "v": torch.tensor(v, dtype=dtype, device=device)}


def gray_scott_benchmark_ic(n: int = 256, dtype=torch.float64, device="cuda"):
    """(u0, v0) interiors of benchmarks/benchmark_gray_scott.py:59-68: 1 - 0.05 U[0,1) and
    0.25 + 0.05 U[0,1) from numpy.random.seed(42), and a 20 x 20 square of (0.5, 0.25) at
    the centre."""
    rs = np.random.RandomState(42)
    u0 = np.ones((n, n)) - 0.5 * rs.rand(n, n) * 0.1
    v0 = 0.25 * np.ones((n, n)) + 0.5 * rs.rand(n, n) * 0.1
    c, r = n // 2, 10
    u0[c - r:c + r, c - r:c + r] = 0.5
    v0[c - r:c + r, c - r:c + r] = 0.25
    return (torch.tensor(u0, dtype=dtype, device=device), torch.tensor(v0, dtype=dtype, device=device))
