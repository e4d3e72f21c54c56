"""Uniform cell-centred grids with ghost cells (host-side geometry only).

Mirrors moljax/core/grid.py:20-259 (``Grid1D``/``Grid2D``: dx = (max-min)/n,
padded shapes (n+2g,) and (ny+2g, nx+2g), y on axis 0) and also accepts the
README spellings ``Grid1D(n=, L=, bc_type=)`` and
``Grid2D(nx=, ny=, Lx=, Ly=, periodic=)`` (README.md:49-52, 89-91).
Coordinates are returned as float64 torch tensors on the CPU.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Tuple, Union

import torch


@dataclass(frozen=True, init=False)
class Grid1D:
    """1D grid; arrays have shape (nx + 2*n_ghost,), interior [n_ghost : nx+n_ghost]."""

    nx: int
    x_min: float
    x_max: float
    n_ghost: int
    bc_type: Optional[str]

    def __init__(self, nx: Optional[int] = None, x_min: float = 0.0, x_max: Optional[float] = None,
                 n_ghost: int = 1, *, n: Optional[int] = None, L: Optional[float] = None,
                 bc_type: Optional[str] = None):
        nx = n if nx is None else nx
        if nx is None:
            raise TypeError("Grid1D needs nx (or n=)")
        if x_max is None:
            x_max = x_min + (1.0 if L is None else float(L))
        object.__setattr__(self, "nx", int(nx))
        object.__setattr__(self, "x_min", float(x_min))
        object.__setattr__(self, "x_max", float(x_max))
        object.__setattr__(self, "n_ghost", int(n_ghost))
        object.__setattr__(self, "bc_type", bc_type)

    @classmethod
    def uniform(cls, nx: int, x_min: float, x_max: float, n_ghost: int = 1) -> "Grid1D":
        return cls(nx, x_min, x_max, n_ghost)

    @property
    def dx(self) -> float:
        return (self.x_max - self.x_min) / self.nx

    @property
    def nx_total(self) -> int:
        return self.nx + 2 * self.n_ghost

    @property
    def interior_slice(self) -> slice:
        return slice(self.n_ghost, self.n_ghost + self.nx)

    @property
    def min_dx(self) -> float:
        return self.dx

    @property
    def min_dx2(self) -> float:
        return self.dx ** 2

    def x_coords(self, include_ghost: bool = False) -> torch.Tensor:
        if include_ghost:
            x0 = self.x_min - self.n_ghost * self.dx
            return torch.linspace(x0 + 0.5 * self.dx, x0 + (self.nx_total - 0.5) * self.dx,
                                  self.nx_total, dtype=torch.float64)
        return torch.linspace(self.x_min + 0.5 * self.dx, self.x_max - 0.5 * self.dx, self.nx,
                              dtype=torch.float64)

    @property
    def x(self) -> torch.Tensor:
        return self.x_coords()


@dataclass(frozen=True, init=False)
class Grid2D:
    """2D grid; arrays have shape (ny+2g, nx+2g), y is axis 0 (rows)."""

    nx: int
    ny: int
    x_min: float
    x_max: float
    y_min: float
    y_max: float
    n_ghost: int
    periodic: Optional[bool]

    def __init__(self, nx: int, ny: Optional[int] = None, x_min: float = 0.0,
                 x_max: Optional[float] = None, y_min: float = 0.0, y_max: Optional[float] = None,
                 n_ghost: int = 1, *, Lx: Optional[float] = None, Ly: Optional[float] = None,
                 periodic: Optional[bool] = None):
        ny = nx if ny is None else ny
        if x_max is None:
            x_max = x_min + (1.0 if Lx is None else float(Lx))
        if y_max is None:
            y_max = y_min + (1.0 if Ly is None else float(Ly))
        object.__setattr__(self, "nx", int(nx))
        object.__setattr__(self, "ny", int(ny))
        object.__setattr__(self, "x_min", float(x_min))
        object.__setattr__(self, "x_max", float(x_max))
        object.__setattr__(self, "y_min", float(y_min))
        object.__setattr__(self, "y_max", float(y_max))
        object.__setattr__(self, "n_ghost", int(n_ghost))
        object.__setattr__(self, "periodic", periodic)

    @classmethod
    def uniform(cls, nx, ny, x_min, x_max, y_min, y_max, n_ghost=1) -> "Grid2D":
        return cls(nx, ny, x_min, x_max, y_min, y_max, n_ghost)

    @property
    def dx(self) -> float:
        return (self.x_max - self.x_min) / self.nx

    @property
    def dy(self) -> float:
        return (self.y_max - self.y_min) / self.ny

    @property
    def nx_total(self) -> int:
        return self.nx + 2 * self.n_ghost

    @property
    def ny_total(self) -> int:
        return self.ny + 2 * self.n_ghost

    @property
    def interior_slice(self) -> Tuple[slice, slice]:
        g = self.n_ghost
        return (slice(g, g + self.ny), slice(g, g + self.nx))

    @property
    def min_dx(self) -> float:
        return min(self.dx, self.dy)

    @property
    def min_dx2(self) -> float:
        return self.min_dx ** 2

    def meshgrid(self, include_ghost: bool = False):
        """(X, Y) with X varying along columns (moljax/core/grid.py:220-259)."""
        if include_ghost:
            x0 = self.x_min - self.n_ghost * self.dx
            y0 = self.y_min - self.n_ghost * self.dy
            x = torch.linspace(x0 + 0.5 * self.dx, x0 + (self.nx_total - 0.5) * self.dx,
                               self.nx_total, dtype=torch.float64)
            y = torch.linspace(y0 + 0.5 * self.dy, y0 + (self.ny_total - 0.5) * self.dy,
                               self.ny_total, dtype=torch.float64)
        else:
            x = torch.linspace(self.x_min + 0.5 * self.dx, self.x_max - 0.5 * self.dx, self.nx,
                               dtype=torch.float64)
            y = torch.linspace(self.y_min + 0.5 * self.dy, self.y_max - 0.5 * self.dy, self.ny,
                               dtype=torch.float64)
        Y, X = torch.meshgrid(y, x, indexing="ij")
        return X, Y

    @property
    def x(self) -> torch.Tensor:
        return self.meshgrid()[0]

    @property
    def y(self) -> torch.Tensor:
        return self.meshgrid()[1]


GridType = Union[Grid1D, Grid2D]
