"""Oracle: grids, ghost-cell BCs, FD stencils, reactions, FFT symbols, Helmholtz.

TEST INFRASTRUCTURE ONLY (see ``oracle/__init__.py``).  NumPy FP64
restatement of the reference; padded arrays with ghost cells exactly as the
reference stores them (y is axis 0, x is axis 1).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

PERIODIC, DIRICHLET, NEUMANN = 0, 1, 2  # moljax/core/bc.py:26-30


# ---------------------------------------------------------------- grids
@dataclass(frozen=True)
class Grid1D:
    """moljax/core/grid.py:20-112 (cell-centred, dx=(max-min)/nx)."""
    nx: int
    x_min: float
    x_max: float
    n_ghost: int = 1

    @property
    def dx(self):
        return (self.x_max - self.x_min) / self.nx

    @property
    def nx_total(self):
        return self.nx + 2 * self.n_ghost

    @property
    def interior_slice(self):
        return slice(self.n_ghost, self.n_ghost + self.nx)

    def x_coords(self, include_ghost=False):
        """moljax/core/grid.py:89-112."""
        if include_ghost:
            x0 = self.x_min - self.n_ghost * self.dx
            return np.linspace(x0 + 0.5 * self.dx, x0 + (self.nx_total - 0.5) * self.dx,
                               self.nx_total)
        return np.linspace(self.x_min + 0.5 * self.dx, self.x_max - 0.5 * self.dx, self.nx)


@dataclass(frozen=True)
class Grid2D:
    """moljax/core/grid.py:115-259."""
    nx: int
    ny: int
    x_min: float
    x_max: float
    y_min: float
    y_max: float
    n_ghost: int = 1

    @property
    def dx(self):
        return (self.x_max - self.x_min) / self.nx

    @property
    def dy(self):
        return (self.y_max - self.y_min) / self.ny

    @property
    def nx_total(self):
        return self.nx + 2 * self.n_ghost

    @property
    def ny_total(self):
        return self.ny + 2 * self.n_ghost

    @property
    def interior_slice(self):
        g = self.n_ghost
        return (slice(g, g + self.ny), slice(g, g + self.nx))

    @property
    def min_dx(self):
        return min(self.dx, self.dy)

    def meshgrid(self, include_ghost=False):
        """moljax/core/grid.py:220-259 (indexing='xy')."""
        if include_ghost:
            x0 = self.x_min - self.n_ghost * self.dx
            y0 = self.y_min - self.n_ghost * self.dy
            x = np.linspace(x0 + 0.5 * self.dx, x0 + (self.nx_total - 0.5) * self.dx, self.nx_total)
            y = np.linspace(y0 + 0.5 * self.dy, y0 + (self.ny_total - 0.5) * self.dy, self.ny_total)
        else:
            x = np.linspace(self.x_min + 0.5 * self.dx, self.x_max - 0.5 * self.dx, self.nx)
            y = np.linspace(self.y_min + 0.5 * self.dy, self.y_max - 0.5 * self.dy, self.ny)
        return np.meshgrid(x, y, indexing="xy")


def interior(f, grid):
    return f[grid.interior_slice]


def embed(u_int, grid, template):
    out = np.array(template, dtype=np.float64, copy=True)
    out[grid.interior_slice] = u_int
    return out


def pad(u_int, grid):
    """Interior -> padded array with zero ghosts (state.py:268-295)."""
    if isinstance(grid, Grid1D):
        out = np.zeros(grid.nx_total)
    else:
        out = np.zeros((grid.ny_total, grid.nx_total))
    out[grid.interior_slice] = u_int
    return out


# ---------------------------------------------------------------- BCs
def bc_1d(f, grid, kind, left=0.0, right=0.0):
    """moljax/core/bc.py:85-158: periodic wrap, Dirichlet 2b-u, Neumann u -/+ 2dx q."""
    f = np.array(f, dtype=np.float64, copy=True)
    g, nx = grid.n_ghost, grid.nx
    if kind == PERIODIC:
        f[:g] = f[nx:nx + g]
        f[nx + g:] = f[g:2 * g]
    elif kind == DIRICHLET:
        for i in range(g):
            f[g - 1 - i] = 2.0 * left - f[g + i]
            f[nx + g + i] = 2.0 * right - f[nx + g - 1 - i]
    elif kind == NEUMANN:
        for i in range(g):
            f[g - 1 - i] = f[g + i] - 2.0 * grid.dx * left
            f[nx + g + i] = f[nx + g - 1 - i] + 2.0 * grid.dx * right
    else:
        raise ValueError(kind)
    return f


def bc_2d(f, grid, kind, values=None):
    """moljax/core/bc.py:202-307.  x (columns) first, then y (rows)."""
    f = np.array(f, dtype=np.float64, copy=True)
    g, nx, ny = grid.n_ghost, grid.nx, grid.ny
    v = {"left": 0.0, "right": 0.0, "bottom": 0.0, "top": 0.0}
    if values:
        v.update(values)
    if kind == PERIODIC:
        f[:, :g] = f[:, nx:nx + g]
        f[:, nx + g:] = f[:, g:2 * g]
        f[:g, :] = f[ny:ny + g, :]
        f[ny + g:, :] = f[g:2 * g, :]
    elif kind == DIRICHLET:
        for i in range(g):
            f[:, g - 1 - i] = 2.0 * v["left"] - f[:, g + i]
            f[:, nx + g + i] = 2.0 * v["right"] - f[:, nx + g - 1 - i]
        for i in range(g):
            f[g - 1 - i, :] = 2.0 * v["bottom"] - f[g + i, :]
            f[ny + g + i, :] = 2.0 * v["top"] - f[ny + g - 1 - i, :]
    elif kind == NEUMANN:
        for i in range(g):
            f[:, g - 1 - i] = f[:, g + i] - 2.0 * grid.dx * v["left"]
            f[:, nx + g + i] = f[:, nx + g - 1 - i] + 2.0 * grid.dx * v["right"]
        for i in range(g):
            f[g - 1 - i, :] = f[g + i, :] - 2.0 * grid.dy * v["bottom"]
            f[ny + g + i, :] = f[ny + g - 1 - i, :] + 2.0 * grid.dy * v["top"]
    else:
        raise ValueError(kind)
    return f


def apply_bc(state, grid, kinds):
    """moljax/core/bc.py:358-404 with homogeneous values; kinds: name -> BC kind."""
    fn = bc_1d if isinstance(grid, Grid1D) else bc_2d
    return {k: (fn(f, grid, kinds[k]) if k in kinds else f) for k, f in state.items()}


# ---------------------------------------------------------------- stencils
def d1_upwind_1d(f, v, grid):
    """moljax/core/operators.py:64-110 (v>=0 backward, else forward; ghosts zero)."""
    g, nx, dx = grid.n_ghost, grid.nx, grid.dx
    out = np.zeros_like(f, dtype=np.float64)
    bwd = (f[g:g + nx] - f[g - 1:g + nx - 1]) / dx
    fwd = (f[g + 1:g + nx + 1] - f[g:g + nx]) / dx
    vi = v if np.ndim(v) == 0 else np.asarray(v)[g:g + nx]
    out[g:g + nx] = np.where(vi >= 0, bwd, fwd)
    return out


def d1_central_1d(f, grid):
    """moljax/core/operators.py:35-61."""
    g, nx, dx = grid.n_ghost, grid.nx, grid.dx
    out = np.zeros_like(f, dtype=np.float64)
    out[g:g + nx] = (f[g + 1:g + nx + 1] - f[g - 1:g + nx - 1]) / (2.0 * dx)
    return out


def laplacian_1d(f, grid):
    """moljax/core/operators.py:113-152."""
    g, nx = grid.n_ghost, grid.nx
    out = np.zeros_like(f, dtype=np.float64)
    out[g:g + nx] = (f[g + 1:g + nx + 1] - 2.0 * f[g:g + nx] + f[g - 1:g + nx - 1]) / grid.dx ** 2
    return out


def laplacian_2d(f, grid):
    """moljax/core/operators.py:271-322 (d2/dy2 + d2/dx2 on interior, ghosts zero)."""
    g, nx, ny = grid.n_ghost, grid.nx, grid.ny
    out = np.zeros_like(f, dtype=np.float64)
    c = f[g:g + ny, g:g + nx]
    dyy = (f[g + 1:g + ny + 1, g:g + nx] - 2.0 * c + f[g - 1:g + ny - 1, g:g + nx]) / grid.dy ** 2
    dxx = (f[g:g + ny, g + 1:g + nx + 1] - 2.0 * c + f[g:g + ny, g - 1:g + nx - 1]) / grid.dx ** 2
    out[g:g + ny, g:g + nx] = dyy + dxx
    return out


def d1_upwind_2d(f, v, grid, axis):
    """moljax/core/operators.py:200-268."""
    g, nx, ny = grid.n_ghost, grid.nx, grid.ny
    out = np.zeros_like(f, dtype=np.float64)
    c = f[g:g + ny, g:g + nx]
    if axis == 0:
        bwd = (c - f[g - 1:g + ny - 1, g:g + nx]) / grid.dy
        fwd = (f[g + 1:g + ny + 1, g:g + nx] - c) / grid.dy
    else:
        bwd = (c - f[g:g + ny, g - 1:g + nx - 1]) / grid.dx
        fwd = (f[g:g + ny, g + 1:g + nx + 1] - c) / grid.dx
    vi = v if np.ndim(v) == 0 else np.asarray(v)[g:g + ny, g:g + nx]
    out[g:g + ny, g:g + nx] = np.where(vi >= 0, bwd, fwd)
    return out


# ---------------------------------------------------------------- reactions
def gray_scott_reaction(state, F, k):
    """moljax/core/operators.py:644-667: u: -uv^2 + F(1-u); v: uv^2 - (F+k)v."""
    u, v = state["u"], state["v"]
    uvv = u * v * v
    return {"u": -uvv + F * (1.0 - u), "v": uvv - (F + k) * v}


def fisher_kpp_reaction(state, r, name="u"):
    """moljax/core/operators.py:680-705: r u (1-u)."""
    out = {k: np.zeros_like(f) for k, f in state.items()}
    out[name] = r * state[name] * (1.0 - state[name])
    return out


# ---------------------------------------------------------------- symbols
def fd_symbol_1d(n, d):
    """moljax/core/fft_solvers.py:97-121: (2cos(k d) - 2)/d^2, k=2pi fftfreq(n, d)."""
    k = 2.0 * np.pi * np.fft.fftfreq(n, d=d)
    return (2.0 * np.cos(k * d) - 2.0) / (d * d)


def fd_symbol_2d(ny, nx, dy, dx):
    """moljax/core/fft_solvers.py:124-154 (shape (ny, nx))."""
    return fd_symbol_1d(nx, dx)[None, :] + fd_symbol_1d(ny, dy)[:, None]


def spectral_symbol_1d(n, d):
    """Pseudo-spectral -k^2 (benchmarks/benchmark_vs_scipy.py:77-80)."""
    k = 2.0 * np.pi * np.fft.fftfreq(n, d=d)
    return -(k * k)


def spectral_symbol_2d(ny, nx, dy, dx):
    return spectral_symbol_1d(nx, dx)[None, :] + spectral_symbol_1d(ny, dy)[:, None]


# ---------------------------------------------------------------- Helmholtz
_fft2, _ifft2 = np.fft.fft2, np.fft.ifft2


def set_fft_workers(workers):
    """Use scipy.fft with `workers` threads (CPU baseline timing); None restores numpy.fft."""
    global _fft2, _ifft2
    if workers is None:
        _fft2, _ifft2 = np.fft.fft2, np.fft.ifft2
        return
    import scipy.fft as sf
    _fft2 = lambda a: sf.fft2(a, workers=workers)  # noqa: E731
    _ifft2 = lambda a: sf.ifft2(a, workers=workers)  # noqa: E731


def helmholtz_denominator(lam, dt, D):
    """moljax/core/fft_solvers.py:244-248 / 281-285 (|denom|<1e-14 -> 1e-14)."""
    denom = 1.0 - dt * D * lam
    return np.where(np.abs(denom) < 1e-14, 1e-14, denom)


def solve_helmholtz_1d(rhs, lam, dt, D):
    """moljax/core/fft_solvers.py:222-258."""
    return np.fft.ifft(np.fft.fft(rhs) / helmholtz_denominator(lam, dt, D)).real


def solve_helmholtz_2d(rhs, lam, dt, D):
    """moljax/core/fft_solvers.py:261-294: ifft2(fft2(rhs)/(1 - dt D lam)).real."""
    return _ifft2(_fft2(rhs) / helmholtz_denominator(lam, dt, D)).real


def apply_diffusion_inverse_fft(state, grid, dt, diffusivities, lam):
    """moljax/core/fft_solvers.py:406-445 with solve_diffusion_fft_field 368-399.

    Each field with D > 1e-14 is solved on the interior and embedded back into
    the padded array (ghosts keep the input's values); others pass through.
    """
    solve = solve_helmholtz_1d if isinstance(grid, Grid1D) else solve_helmholtz_2d
    out = {}
    for name, f in state.items():
        D = diffusivities.get(name, 0.0)
        if D > 1e-14:
            out[name] = embed(solve(interior(f, grid), lam, dt, D), grid, f)
        else:
            out[name] = f
    return out


# ---------------------------------------------------------------- norms
def scaled_error_norm(err, y, grid, atol, rtol):
    """moljax/core/state.py:312-343: sqrt(sum((e/(atol+rtol|y|))^2)/n_dof) over interiors."""
    tot = 0.0
    n = 0
    for k in err:
        e = interior(err[k], grid)
        s = atol + rtol * np.abs(interior(y[k], grid))
        tot += float(np.sum((e / s) ** 2))
        n += e.size
    return float(np.sqrt(tot / n))


def is_finite(state):
    """moljax/core/utils.py:186-197 (all entries, ghosts included)."""
    return all(bool(np.all(np.isfinite(f))) for f in state.values())


# ---------------------------------------------------------------- initial data
def gray_scott_ic(grid, seed, noise=0.01, frac=0.1):
    """examples/gray_scott_2d.py:42-73 on the padded grid.

    u=1, v=0 except the central square |x-cx|<frac*Lx, |y-cy|<frac*Ly where
    u=0.5, v=0.25; plus noise*U[-1,1].  The reference draws the noise from
    jax.random.PRNGKey(42); this restatement draws it from
    numpy.random.default_rng(seed) (JAX streams are not reproducible here).
    """
    X, Y = grid.meshgrid(include_ghost=True)
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
    return {"u": u, "v": v}
