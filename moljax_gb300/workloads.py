"""Seeded synthetic workloads (initial data for the benchmark configurations).

``gray_scott_initial_condition`` restates the Gray-Scott initial condition of
examples/gray_scott_2d.py:42-73: u = 1, v = 0 except the central square
|x-cx| < 0.1 Lx, |y-cy| < 0.1 Ly where u = 0.5, v = 0.25, plus 0.01*U[-1,1]
noise on the padded arrays.  The reference draws the noise from
jax.random.PRNGKey(42); here it comes from numpy.random.default_rng(seed).
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
