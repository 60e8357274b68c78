"""Yee grid with the reference's semantics (core/grid.py).

``GridSpec`` and ``YeeGrid`` keep the reference's names, arguments and quirks:
sizes from ``ceil(L * resolution)`` (grid.py:96-100), boundary layers added
outside the physical size (grid.py:107-111), component shapes (grid.py:157-168),
``point_to_index`` clamping to the *physical* count (grid.py:350-352) and the
``np.ix_`` regions of ``get_component_indices`` (grid.py:383-513).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Literal, Union

import numpy as np

C0 = 299792458.0


@dataclass
class GridSpec:
    """core/grid.py:16-50."""

    size: tuple
    resolution: Union[float, tuple]
    boundary_layers: int = 10

    def __post_init__(self):
        if any(s < 0 for s in self.size):
            raise ValueError("Grid size components must be non-negative")
        if isinstance(self.resolution, (int, float)):
            self.resolution = (self.resolution, self.resolution, self.resolution)
        elif len(self.resolution) != 3:
            raise ValueError("Resolution must be scalar or 3-tuple")
        if any(r <= 0 for r in self.resolution):
            raise ValueError("Resolution must be positive")


class YeeGrid:
    """core/grid.py:53-522."""

    def __init__(self, spec: GridSpec):
        self.spec = spec
        self._setup_grid()

    @classmethod
    def from_total(cls, dims, d: float, layers: int) -> "YeeGrid":
        """Grid whose total size (boundary layers included) is ``dims``; the
        physical size is set half a cell short of the integer so that the
        ``ceil`` of grid.py:96 lands on ``n - 2*layers``."""
        nx, ny = int(dims[0]), int(dims[1])
        nz = int(dims[2]) if len(dims) > 2 else 1
        lz = 0.0 if nz <= 1 else (nz - 2 * layers - 0.5) * d
        g = cls(GridSpec(size=((nx - 2 * layers - 0.5) * d, (ny - 2 * layers - 0.5) * d, lz),
                         resolution=1.0 / d, boundary_layers=layers))
        if g.dimensions != (nx, ny, max(nz, 1)):
            raise ValueError(f"cannot realise total dims {dims} (got {g.dimensions})")
        return g

    def _setup_grid(self):
        self.Lx, self.Ly, self.Lz = self.spec.size
        self.res_x, self.res_y, self.res_z = self.spec.resolution
        self.dx = 1.0 / self.res_x if self.res_x > 0 else 0.0
        self.dy = 1.0 / self.res_y if self.res_y > 0 else 0.0
        self.dz = 1.0 / self.res_z if self.res_z > 0 else 0.0
        self.is_2d = self.Lz == 0.0
        self.is_3d = not self.is_2d
        self.Nx = int(np.ceil(self.Lx * self.res_x)) if self.Lx > 0 else 1
        self.Ny = int(np.ceil(self.Ly * self.res_y)) if self.Ly > 0 else 1
        self.Nz = int(np.ceil(self.Lz * self.res_z)) if self.Lz > 0 and not self.is_2d else 1
        if self.is_2d:
            self.Nz = 1
            self.dz = 0.0
        self.pml_layers = self.spec.boundary_layers
        self.Nx_total = self.Nx + 2 * self.pml_layers
        self.Ny_total = self.Ny + 2 * self.pml_layers
        self.Nz_total = self.Nz + (2 * self.pml_layers if not self.is_2d else 0)
        self.origin = np.array([-self.pml_layers * self.dx, -self.pml_layers * self.dy,
                                -self.pml_layers * self.dz if not self.is_2d else 0.0])

    @property
    def dimensions(self):
        return (self.Nx_total, self.Ny_total, self.Nz_total)

    @property
    def physical_dimensions(self):
        return (self.Nx, self.Ny, self.Nz)

    @property
    def spacing(self):
        return (self.dx, self.dy, self.dz)

    def get_field_shape(self, component: Literal["Ex", "Ey", "Ez", "Hx", "Hy", "Hz"]):
        nx, ny, nz = self.dimensions
        if component == "Ex":
            shape = (nx, ny - 1, nz - 1) if not self.is_2d else (nx, ny - 1)
        elif component == "Ey":
            shape = (nx - 1, ny, nz - 1) if not self.is_2d else (nx - 1, ny)
        elif component == "Ez":
            shape = (nx - 1, ny - 1, nz) if not self.is_2d else (nx - 1, ny - 1)
        elif component == "Hx":
            shape = (nx - 1, ny, nz) if not self.is_2d else (nx - 1, ny)
        elif component == "Hy":
            shape = (nx, ny - 1, nz) if not self.is_2d else (nx, ny - 1)
        elif component == "Hz":
            shape = (nx, ny, nz - 1) if not self.is_2d else (nx, ny)
        else:
            raise ValueError(f"Unknown field component: {component}")
        return shape

    def get_coordinates(self, component):
        x = self.origin[0] + np.arange(self.Nx_total) * self.dx
        y = self.origin[1] + np.arange(self.Ny_total) * self.dy
        z = self.origin[2] + np.arange(self.Nz_total) * self.dz
        if component in ["Ey", "Ez", "Hy", "Hz"]:
            x = x[:-1] + self.dx / 2
        if component in ["Ex", "Ez", "Hx", "Hz"]:
            y = y[:-1] + self.dy / 2
        if component in ["Ex", "Ey", "Hx", "Hy"] and not self.is_2d:
            z = z[:-1] + self.dz / 2
        return (x, y) if self.is_2d else (x, y, z)

    def is_inside_pml(self, i, j, k=0):
        p = self.pml_layers
        if i < p or i >= self.Nx_total - p:
            return True
        if j < p or j >= self.Ny_total - p:
            return True
        return (not self.is_2d) and (k < p or k >= self.Nz_total - p)

    def get_physical_indices(self):
        p = self.pml_layers
        return (slice(p, self.Nx_total - p), slice(p, self.Ny_total - p),
                slice(p, self.Nz_total - p) if not self.is_2d else slice(None))

    def _inv_sq(self):
        inv = (1 / self.dx) ** 2 + (1 / self.dy) ** 2
        if not self.is_2d:
            inv += (1 / self.dz) ** 2
        return inv

    def get_courant_number(self, dt: float) -> float:
        return C0 * dt * np.sqrt(self._inv_sq())

    def get_time_step(self, safety_factor: float = 0.9) -> float:
        return self.suggest_time_step(safety_factor)

    def suggest_time_step(self, safety_factor: float = 0.9) -> float:
        return safety_factor / (C0 * np.sqrt(self._inv_sq()))

    def point_to_index(self, point):
        x, y, z = point
        i = int(round((x - self.origin[0]) / self.dx))
        j = int(round((y - self.origin[1]) / self.dy))
        k = int(round((z - self.origin[2]) / self.dz)) if self.is_3d else 0
        i = max(0, min(i, self.Nx - 1))
        j = max(0, min(j, self.Ny - 1))
        k = max(0, min(k, self.Nz - 1))
        return (i, j, k)

    def index_to_coord(self, dim, indices):
        if dim not in (0, 1, 2):
            raise ValueError(f"Invalid dimension: {dim}. Must be 0, 1, or 2.")
        return self.origin[dim] + indices * self.spacing[dim]

    def get_component_indices(self, component, x_min, x_max, y_min, y_max, z_min, z_max):
        x_min = max(0, min(x_min, self.Nx - 1))
        x_max = max(1, min(x_max, self.Nx))
        y_min = max(0, min(y_min, self.Ny - 1))
        y_max = max(1, min(y_max, self.Ny))
        if self.is_3d:
            z_min = max(0, min(z_min, self.Nz - 1))
            z_max = max(1, min(z_max, self.Nz))
        else:
            z_min, z_max = 0, 1
        if component not in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
            raise ValueError(f"Invalid field component: {component}")
        shape = self.get_field_shape(component)
        xr = range(x_min, min(x_max, shape[0]))
        yr = range(y_min, min(y_max, shape[1]))
        if self.is_2d:
            return np.ix_(xr, yr)
        return np.ix_(xr, yr, range(z_min, min(z_max, shape[2])))

    def region_bounds(self, center, size):
        """Index bounds of a (center, size) region (sources/base.py:97-139)."""
        h = [s / 2 for s in size]
        x0, y0, z0 = self.point_to_index((center[0] - h[0], center[1] - h[1], center[2] - h[2]))
        x1, y1, z1 = self.point_to_index((center[0] + h[0], center[1] + h[1], center[2] + h[2]))
        if x0 == x1:
            x1 = x0 + 1
        if y0 == y1:
            y1 = y0 + 1
        if z0 == z1 and self.is_3d:
            z1 = z0 + 1
        return x0, x1, y0, y1, z0, z1

    def __repr__(self):
        d = "2D" if self.is_2d else "3D"
        return (f"YeeGrid({d}, shape={self.dimensions}, spacing=({self.dx:.2e}, {self.dy:.2e}, {self.dz:.2e}), "
                f"PML={self.pml_layers})")
