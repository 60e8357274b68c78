"""MaxwellUpdater / FDTDSolver with the reference interface (core/solver.py), on
the native stepper.

``MaxwellUpdater(grid, dt, material_arrays)`` builds the update coefficients on
the device (core/solver.py:113-133, 458-533) and ``step(fields)`` advances H then
E through libprismo_cuda.  Extensions (keyword-only): ``pml`` (CPML thickness or
PMLParams), ``mode`` ("corrected" or "legacy": the reference's own stepper,
core/solver.py:167-456, reproduced exactly in float64), ``sched`` and
``precision``.
"""

from __future__ import annotations

from typing import Optional, Union

import numpy as np

from .backend import CudaBackend, DeviceArray, resolve
from .engine import FDTDEngine
from .fields import ElectromagneticFields
from .pml import PMLParams

EPS0 = 8.854187817e-12
C0 = 299792458.0


def _pml_params(pml) -> Optional[PMLParams]:
    if pml is None or pml is False:
        return None
    if isinstance(pml, PMLParams):
        return pml if pml.thickness > 0 else None
    t = int(pml)
    return PMLParams(thickness=t) if t > 0 else None


class MaxwellUpdater:
    """core/solver.py:24-568 on the device."""

    def __init__(self, grid, dt: float, material_arrays: Optional[dict] = None, backend=None, *,
                 pml: Union[int, PMLParams, None] = None, mode: str = "corrected", sched: str = "auto",
                 precision: Optional[str] = None):
        self.grid = grid
        self.dt = dt
        self.backend = resolve(backend)
        if not isinstance(self.backend, CudaBackend):
            raise TypeError("this MaxwellUpdater runs on the cuda backend")
        self.eps0 = EPS0
        self.mu0 = 4 * self.backend.pi * 1e-7
        self.c = C0
        courant = grid.get_courant_number(dt)
        if courant >= 1.0:  # core/solver.py:67-72
            raise ValueError(f"Time step dt={dt:.2e} violates Courant condition (S={courant:.3f} >= 1)")
        nx, ny, nz = grid.dimensions
        ma = dict(material_arrays or {})
        torch = __import__("torch")

        def dev(name, default):
            v = ma.get(name)
            if v is None:
                return DeviceArray(torch.full((nx, ny, nz), default, dtype=torch.float64, device=self.backend.device))
            if isinstance(v, DeviceArray):
                return DeviceArray(v.tensor.to(torch.float64))
            return self.backend.asarray(np.asarray(v, dtype=np.float64))

        self.eps_rel = dev("eps_rel", 1.0)
        self.mu_rel = dev("mu_rel", 1.0)
        self.sigma_e = dev("sigma_e", 0.0)
        self.sigma_m = dev("sigma_m", 0.0)
        self.dx, self.dy, self.dz = grid.spacing
        self.pml = _pml_params(pml)
        self.mode = mode
        self.precision = precision or self.backend.precision
        self.engine = FDTDEngine(grid.dimensions, grid.spacing, dt, is_2d=grid.is_2d, precision=self.precision,
                                 mode=mode, sched=sched, material_arrays={
                                     k: getattr(self, k).tensor for k in ("eps_rel", "mu_rel", "sigma_e", "sigma_m")
                                     if k in ma},
                                 pml=self.pml, device=str(self.backend.device), bind_later=True)

    # cell-centred coefficients of core/solver.py:113-133 (computed on demand)
    def _cell(self):
        e = self.eps0 * self.eps_rel.tensor
        s = self.sigma_e.tensor * self.dt / (2 * e)
        mu = self.mu0 * self.mu_rel.tensor
        sm = self.sigma_m.tensor * self.dt / (2 * mu)
        return (1 - s) / (1 + s), (self.dt / e) / (1 + s), (1 - sm) / (1 + sm), (self.dt / mu) / (1 + sm)

    @property
    def Ca(self): return DeviceArray(self._cell()[0])
    @property
    def Cb(self): return DeviceArray(self._cell()[1])
    @property
    def Da(self): return DeviceArray(self._cell()[2])
    @property
    def Db(self): return DeviceArray(self._cell()[3])

    def step(self, fields: ElectromagneticFields, amps=None) -> None:
        """One leap-frog step (core/solver.py:535-552): H^{n+1/2} then E^{n+1}."""
        fields._bind(self.engine)
        self.engine.step(1, amps)

    def run_steps(self, fields: ElectromagneticFields, n: int, amps=None) -> None:
        fields._bind(self.engine)
        self.engine.step(int(n), amps)

    def update_magnetic_fields(self, fields):
        raise NotImplementedError("the device stepper advances H and E together; call step()")

    def update_electric_fields(self, fields):
        raise NotImplementedError("the device stepper advances H and E together; call step()")

    def get_time_step(self) -> float:
        return self.dt

    def get_courant_number(self) -> float:
        return self.grid.get_courant_number(self.dt)

    def __repr__(self):
        return f"MaxwellUpdater(dt={self.dt:.2e}s, Courant={self.get_courant_number():.3f}, grid={self.grid.dimensions})"


class FDTDSolver:
    """core/solver.py:571-704 on the device."""

    def __init__(self, grid, dt: Optional[float] = None, material_arrays: Optional[dict] = None, backend=None, *,
                 pml=None, mode: str = "corrected", sched: str = "auto", precision: Optional[str] = None):
        self.grid = grid
        self.backend = resolve(backend)
        if dt is None:
            dt = grid.suggest_time_step(safety_factor=0.95)
        self.fields = ElectromagneticFields(grid, backend=self.backend,
                                            dtype=None if precision is None else
                                            (np.float32 if precision == "fp32" else np.float64))
        self.updater = MaxwellUpdater(grid, dt, material_arrays, backend=self.backend, pml=pml, mode=mode,
                                      sched=sched, precision=precision)
        self.time = 0.0
        self.step_count = 0

    def run(self, total_time: float, callback=None) -> None:
        dt = self.updater.get_time_step()
        self.run_steps(int(np.ceil(total_time / dt)), callback)

    def run_steps(self, num_steps: int, callback=None) -> None:
        dt = self.updater.get_time_step()
        if callback is None:
            self.updater.run_steps(self.fields, num_steps)
            for _ in range(num_steps):
                self.time += dt
            self.step_count += num_steps
            return
        for step in range(num_steps):
            self.updater.step(self.fields)
            self.time += dt
            self.step_count += 1
            callback(self, step)

    def step(self, fields: Optional[ElectromagneticFields] = None) -> None:
        self.updater.step(fields if fields is not None else self.fields)
        self.time += self.updater.get_time_step()
        self.step_count += 1

    def reset(self) -> None:
        self.fields.zero_fields()
        for p in self.updater.engine.psi:
            p.zero_()
        self.time = 0.0
        self.step_count = 0

    def get_simulation_info(self) -> dict:
        return {"time": self.time, "step_count": self.step_count, "dt": self.updater.get_time_step(),
                "courant_number": self.updater.get_courant_number(), "grid_dimensions": self.grid.dimensions,
                "is_2d": self.grid.is_2d, "field_energy": self.fields.get_field_energy()}

    def __repr__(self):
        info = self.get_simulation_info()
        return f"FDTDSolver(t={info['time']:.2e}s, steps={info['step_count']}, E_total={info['field_energy']:.2e}J)"
