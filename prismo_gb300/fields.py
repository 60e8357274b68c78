"""Electromagnetic field storage on the device (core/fields.py:20-415 interface).

Storage is one or two padded field sets (see engine.py); each component is a
``DeviceArray`` view with the reference shape (core/grid.py:157-168) that always
resolves to the set holding the current fields, so handles stay valid across the
fused stepper's ping-pong.
"""

from __future__ import annotations

import numpy as np

from .backend import CudaBackend, DeviceArray, resolve
from .engine import COMP_INDEX, COMPONENTS, component_shape, new_field_sets, storage_shape

EPS0 = 8.854187817e-12
MU0 = 4 * np.pi * 1e-7


class ElectromagneticFields:
    """core/fields.py:20-415 on device storage."""

    def __init__(self, grid, dtype=None, backend=None):
        self.grid = grid
        self.backend = resolve(backend)
        if not isinstance(self.backend, CudaBackend):
            raise TypeError("ElectromagneticFields here stores fields for the cuda backend")
        torch = __import__("torch")
        if dtype is None:
            self.tdtype = self.backend.field_dtype
        else:
            self.tdtype = torch.float32 if np.dtype(dtype) == np.float32 else torch.float64
        self.dtype = np.float32 if self.tdtype == torch.float32 else np.float64
        self.dims = grid.dimensions
        self.is_2d = grid.is_2d
        self.buf_shape = storage_shape(self.dims, self.is_2d)
        self._sets = new_field_sets(self.buf_shape, self.tdtype, self.backend.device, 1)
        self._cur = 0
        self._engine = None  # engine currently bound to this storage
        self._fields = {c: DeviceArray(resolver=self._resolver(c)) for c in COMPONENTS}

    # -- storage --------------------------------------------------------------
    def _resolver(self, comp):
        q = COMP_INDEX[comp]
        shp = component_shape(comp, self.dims, self.is_2d)

        def view():
            s = self._sets[self.current_set()]
            if self.is_2d:
                return s[q, : shp[0], : shp[1]]
            return s[q, : shp[0], : shp[1], : shp[2]]

        return view

    def current_set(self) -> int:
        if self._engine is not None:
            return self._engine.cur
        return self._cur

    def _bind(self, engine):
        """Attach this storage to an engine (second set allocated when needed)."""
        if self._engine is engine:
            return
        if self._engine is not None:
            self._cur = self._engine.cur
        engine.bind(self._sets, self._cur)
        self._sets = engine.sets
        self._engine = engine

    # -- reference interface -----------------------------------------------------
    def __getitem__(self, component):
        if component not in self._fields:
            raise KeyError(f"Unknown field component: {component}")
        return self._fields[component]

    def __setitem__(self, component, value):
        if component not in self._fields:
            raise KeyError(f"Unknown field component: {component}")
        arr = self._fields[component]
        if np.isscalar(value):
            arr.fill(value)
            return
        v = value.tensor if isinstance(value, DeviceArray) else np.asarray(value)
        if tuple(v.shape) != arr.shape:
            raise ValueError(f"Shape mismatch for {component}: expected {arr.shape}, got {tuple(v.shape)}")
        arr[...] = value

    @property
    def Ex(self): return self._fields["Ex"]
    @property
    def Ey(self): return self._fields["Ey"]
    @property
    def Ez(self): return self._fields["Ez"]
    @property
    def Hx(self): return self._fields["Hx"]
    @property
    def Hy(self): return self._fields["Hy"]
    @property
    def Hz(self): return self._fields["Hz"]

    def get_field_type_components(self, field_type):
        if field_type == "E":
            return self.Ex, self.Ey, self.Ez
        if field_type == "H":
            return self.Hx, self.Hy, self.Hz
        raise ValueError(f"Unknown field type: {field_type}")

    def zero_fields(self):
        for s in self._sets:
            s.zero_()

    def get_field_energy(self, region=None) -> float:
        """core/fields.py:237-285: 0.5 (eps0 |E|^2 + mu0 |H|^2) dV (vacuum weights)."""
        dx, dy, dz = self.grid.spacing
        dV = dx * dy * (dz if not self.is_2d else 1.0)
        e = h = 0.0
        for c in COMPONENTS:
            t = self._fields[c].tensor
            if region is not None:
                t = t[region]
            v = float((t.double() ** 2).sum().item())
            if c[0] == "E":
                e += v
            else:
                h += v
        return 0.5 * EPS0 * e * dV + 0.5 * MU0 * h * dV

    def get_field_magnitude(self, field_type, region=None):
        fx, fy, fz = (f.tensor for f in self.get_field_type_components(field_type))
        ms = [min(s) for s in zip(fx.shape, fy.shape, fz.shape)]
        sl = tuple(slice(0, m) for m in ms)
        return DeviceArray((fx[sl] ** 2 + fy[sl] ** 2 + fz[sl] ** 2).sqrt())

    def to_numpy(self) -> dict:
        return {c: self._fields[c].to_numpy() for c in COMPONENTS}

    @property
    def nbytes(self):
        return sum(self._fields[c].nbytes for c in COMPONENTS)

    def __repr__(self):
        return f"ElectromagneticFields(grid={self.dims}, dtype={np.dtype(self.dtype).name}, backend=cuda)"
