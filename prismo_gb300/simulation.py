"""Simulation with the reference interface (core/simulation.py:22-250) on the
device engine.

Ordering per step follows core/simulation.py:147-164: H^{n+1/2}, E^{n+1}, time
advances, sources at t_{n+1}, monitors at t_{n+1}.  Known sources (point, plane,
line, TFSF) and DFT monitors run inside the native step; other sources and the
time-domain records are applied from the host on device arrays.  ``run`` advances
in batches of native steps when no per-step host work is needed.

Extensions (keyword-only): ``material_arrays`` (cell-centred eps_rel, mu_rel,
sigma_e, sigma_m, as core/solver.py:79-111 takes them; the reference Simulation
has no material API), ``precision``, ``mode``; ``add_dispersive`` for ADE
regions.  With boundary_conditions="pml" the ``pml_layers`` outside the physical
size carry a CPML (the reference adds the layers but never absorbs in them).
"""

from __future__ import annotations

import time as time_module
from typing import Optional

import numpy as np

from .backend import resolve
from .fields import ElectromagneticFields
from .grid import GridSpec, YeeGrid
from .monitors import FieldMonitor, Monitor
from .solver import FDTDSolver
from .sources import Source, TFSFSource, amplitude_table


class Simulation:
    """core/simulation.py:22-250."""

    BATCH = 1024  # native steps per batched call in run()

    def __init__(self, size, resolution, boundary_conditions: str = "pml", pml_layers: int = 10,
                 courant_factor: float = 0.9, *, material_arrays: Optional[dict] = None, backend=None,
                 precision: Optional[str] = None, mode: str = "corrected", sched: str = "auto"):
        self.grid_spec = GridSpec(size=size, resolution=resolution, boundary_layers=pml_layers)
        self.grid = YeeGrid(self.grid_spec)
        self.size = size
        self.resolution = resolution
        self.boundary_conditions = boundary_conditions
        self.courant_factor = courant_factor
        self.backend = resolve(backend)
        self.dt = self.grid.get_time_step(courant_factor)
        pml = pml_layers if (boundary_conditions == "pml" and mode == "corrected") else None
        self.solver = FDTDSolver(self.grid, self.dt, material_arrays, backend=self.backend, pml=pml, mode=mode,
                                 sched=sched, precision=precision)
        self.fields: ElectromagneticFields = self.solver.fields
        self.engine = self.solver.updater.engine
        self.fields._bind(self.engine)
        self.sources: list = []
        self.monitors: list = []
        self._device_sources: list = []  # sources injected by the native step
        self._host_sources: list = []
        self._tfsf: Optional[TFSFSource] = None
        self.step_count = 0
        self.current_time = 0.0

    # -- setup ---------------------------------------------------------------
    def add_source(self, source: Source) -> None:
        source.initialize(self.grid)
        self.sources.append(source)
        if isinstance(source, TFSFSource):
            if self._tfsf is not None:
                raise ValueError("one TFSF plane per simulation")
            self.engine.set_tfsf(source.plane_index(), source.direction_sign, source.polarization,
                                 source.waveform, eps_b=source.eps_background)
            self._tfsf = source
            return
        if hasattr(source, "injections"):
            for comp, idx, w, _ in source.injections():
                self.engine.add_source(comp, self.engine.offsets(comp, idx),
                                       None if w is None else np.asarray(w).reshape(-1), source.waveform)
            self._device_sources.append(source)
        else:
            self._host_sources.append(source)

    def add_monitor(self, monitor: Monitor) -> None:
        monitor.initialize(self.grid)
        monitor.attach(self.engine, self.current_time + self.dt)
        self.monitors.append(monitor)

    def set_materials(self, material_arrays: dict) -> None:
        """Rebuild the update coefficients from cell-centred material arrays."""
        self.engine._set_materials(material_arrays)

    def add_dispersive(self, material, box) -> None:
        """ADE region: ``box`` = (x0, x1, y0, y1, z0, z1) in E-component indices."""
        regions = list(getattr(self.engine, "ade_regions", []) or [])
        regions.append((box, material.epsilon_inf, material.ade_poles(self.dt)))
        self.engine.set_dispersive(regions)

    # -- stepping --------------------------------------------------------------
    def _times(self, n: int) -> np.ndarray:
        # t_{n+1} by repeated addition, as core/simulation.py:156 accumulates it
        return np.cumsum(np.concatenate([[self.current_time], np.full(n, self.dt)]))[1:]

    def _amps(self, times: np.ndarray):
        cols = []
        if self._device_sources:
            cols.append(amplitude_table(self._device_sources, times))
        if self._tfsf is not None:
            a = self._tfsf.waveform(times) if self._tfsf.enabled else np.zeros(len(times))
            cols.append(np.asarray(a, dtype=np.float64).reshape(-1, 1))
        if not cols:
            return None
        return np.ascontiguousarray(np.concatenate(cols, axis=1))

    def _needs_host_each_step(self) -> bool:
        return bool(self._host_sources) or any(
            not getattr(m, "device_sampled", False) and (not isinstance(m, FieldMonitor) or m.time_domain or
                                                         m._engine is None) for m in self.monitors)

    def step(self) -> None:
        """core/simulation.py:147-164."""
        times = self._times(1)
        self.solver.updater.engine.step(1, self._amps(times))
        self.solver.step_count += 1
        self.step_count += 1
        self.current_time = float(times[-1])
        self.solver.time = self.current_time
        for s in self._host_sources:
            s.update_fields(self.fields, self.current_time, self.dt)
        for m in self.monitors:
            m.update(self.fields, self.current_time, self.dt)

    def run(self, time: float, progress_callback=None, progress_interval: int = 10) -> None:
        """core/simulation.py:107-145."""
        steps = int(np.ceil(time / self.dt))
        start = time_module.time()
        if progress_callback is None and not self._needs_host_each_step():
            done = 0
            while done < steps:
                n = min(self.BATCH, steps - done)
                times = self._times(n)
                self.engine.step(n, self._amps(times))
                for m in self.monitors:
                    if hasattr(m, "_time_steps"):
                        m._time_steps += n
                self.current_time = float(times[-1])
                done += n
            self.step_count += steps
            self.solver.step_count += steps
            self.solver.time = self.current_time
        else:
            for i in range(steps):
                self.step()
                if progress_callback is not None and i % progress_interval == 0:
                    progress_callback(i, steps, self.current_time, time_module.time() - start)
        if progress_callback is not None:
            progress_callback(steps, steps, self.current_time, time_module.time() - start)

    # -- results ---------------------------------------------------------------
    def get_field_data(self, monitor: FieldMonitor, component: str):
        if monitor not in self.monitors:
            raise ValueError("Monitor not found in this simulation")
        return monitor.get_time_data(component)[1]

    def get_frequency_data(self, monitor: FieldMonitor, component: str, frequency: float):
        if monitor not in self.monitors:
            raise ValueError("Monitor not found in this simulation")
        return monitor.get_frequency_data(component, frequency)

    def get_transmission(self, monitor: FieldMonitor, frequency: Optional[float] = None) -> float:
        if monitor not in self.monitors:
            raise ValueError("Monitor not found in this simulation")
        return float(np.mean(monitor.get_power_flow(frequency)))

    def check(self) -> int:
        """Raise on device-side problems (non-finite fields, bounded waits)."""
        return self.engine.check_status()
