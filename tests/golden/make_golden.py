"""Generate golden fixtures by running the reference Prismo package itself.

Run with the path of a checkout of the reference project (read-only):

    python tests/golden/make_golden.py REFERENCE_CHECKOUT

The reference is imported through a harness shim that changes no reference
file: ``builtins.MTLBuffer`` is defined (backends/metal_backend.py:85 annotates
with it unguarded) and a stub ``polars`` module is installed
(io/exporters/parquet_exporter.py:301).  Outputs are small ``.npz`` files
beside this script; the tests read only those files.
"""

from __future__ import annotations

import builtins
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_reference(root: str):
    builtins.MTLBuffer = object
    pl = types.ModuleType("polars")
    pl.DataFrame = object
    sys.modules.setdefault("polars", pl)
    sys.path.insert(0, os.path.join(root, "src"))
    import prismo  # noqa: F401

    prismo.set_backend("numpy")
    return prismo


def rand_fields(rng, grid, comps=("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
    out = {}
    for c in comps:
        shp = grid.get_field_shape(c)
        scale = 1.0 if c.startswith("E") else 1.0 / 377.0
        out[c] = rng.standard_normal(shp) * scale
    return out


def materials(rng, dims, lossy=True):
    eps = rng.uniform(1.0, 12.0, size=dims)
    mu = rng.uniform(1.0, 2.0, size=dims) if lossy else np.ones(dims)
    sig = rng.uniform(0.0, 5e3, size=dims) if lossy else np.zeros(dims)
    sigm = rng.uniform(0.0, 1e3, size=dims) if lossy else np.zeros(dims)
    return {"eps_rel": eps, "mu_rel": mu, "sigma_e": sig, "sigma_m": sigm}


def save(name, **arrays):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **arrays)
    print("wrote", path, sum(np.asarray(v).nbytes for v in arrays.values()), "bytes raw")


def stepper_fixture(prismo, name, size, resolution, layers, nsteps, seed, lossy, corrected=False):
    from prismo.core.fields import ElectromagneticFields
    from prismo.core.grid import GridSpec, YeeGrid
    from prismo.core.solver import MaxwellUpdater

    rng = np.random.default_rng(seed)
    grid = YeeGrid(GridSpec(size=size, resolution=resolution, boundary_layers=layers))
    dt = grid.suggest_time_step(safety_factor=0.5)
    mats = materials(rng, grid.dimensions, lossy)
    cls = corrected_updater(MaxwellUpdater) if corrected else MaxwellUpdater
    up = cls(grid, dt, mats)
    f = ElectromagneticFields(grid)
    init = rand_fields(rng, grid)
    for c, v in init.items():
        f[c] = v
    for _ in range(nsteps):
        up.step(f)
    arrays = {f"init_{c}": v for c, v in init.items()}
    arrays.update({f"out_{c}": np.asarray(f[c]) for c in init})
    arrays.update({k: v for k, v in mats.items()})
    arrays["meta"] = np.array(json.dumps({
        "size": size, "resolution": resolution, "layers": layers, "nsteps": nsteps,
        "dt": dt, "dims": grid.dimensions, "corrected": corrected,
    }))
    save(name, **arrays)


def corrected_updater(base):
    """The reference ``MaxwellUpdater`` with only the H destination slices moved to
    ``[..., 1:-1, ...]`` and the two 2D Ez-family H signs flipped.  Coefficients,
    interpolation and the E update are the reference's own methods."""

    class Corrected(base):
        def _update_h_fields_3d(self, fields):
            Ex, Ey, Ez = fields.Ex, fields.Ey, fields.Ez
            Hx, Hy, Hz = fields.Hx, fields.Hy, fields.Hz
            i = slice(1, -1)
            da, db = self._interpolate_to_hx_points(self.Da), self._interpolate_to_hx_points(self.Db)
            cy = (Ez[:, 1:, 1:-1] - Ez[:, :-1, 1:-1]) / self.dy
            cz = (Ey[:, 1:-1, 1:] - Ey[:, 1:-1, :-1]) / self.dz
            Hx[:, i, i] = da[:, i, i] * Hx[:, i, i] - db[:, i, i] * (cy - cz)
            da, db = self._interpolate_to_hy_points(self.Da), self._interpolate_to_hy_points(self.Db)
            cz = (Ex[1:-1, :, 1:] - Ex[1:-1, :, :-1]) / self.dz
            cx = (Ez[1:, :, 1:-1] - Ez[:-1, :, 1:-1]) / self.dx
            Hy[i, :, i] = da[i, :, i] * Hy[i, :, i] - db[i, :, i] * (cz - cx)
            da, db = self._interpolate_to_hz_points(self.Da), self._interpolate_to_hz_points(self.Db)
            cx = (Ey[1:, 1:-1, :] - Ey[:-1, 1:-1, :]) / self.dx
            cy = (Ex[1:-1, 1:, :] - Ex[1:-1, :-1, :]) / self.dy
            Hz[i, i, :] = da[i, i, :] * Hz[i, i, :] - db[i, i, :] * (cx - cy)

        def _update_h_fields_2d(self, fields):
            Ex, Ey, Ez = fields.Ex, fields.Ey, fields.Ez
            Hx, Hy, Hz = fields.Hx, fields.Hy, fields.Hz
            i = slice(1, -1)
            da = self._interpolate_to_hx_points_2d(self.Da[:, :, 0])
            db = self._interpolate_to_hx_points_2d(self.Db[:, :, 0])
            Hx[:, i] = da[:, i] * Hx[:, i] - db[:, i] * ((Ez[:, 1:] - Ez[:, :-1]) / self.dy)
            da = self._interpolate_to_hy_points_2d(self.Da[:, :, 0])
            db = self._interpolate_to_hy_points_2d(self.Db[:, :, 0])
            Hy[i, :] = da[i, :] * Hy[i, :] + db[i, :] * ((Ez[1:, :] - Ez[:-1, :]) / self.dx)
            da = self._interpolate_to_hz_points_2d(self.Da[:, :, 0])
            db = self._interpolate_to_hz_points_2d(self.Db[:, :, 0])
            cx = (Ey[1:, 1:-1] - Ey[:-1, 1:-1]) / self.dx
            cy = (Ex[1:-1, 1:] - Ex[1:-1, :-1]) / self.dy
            Hz[i, i] = da[i, i] * Hz[i, i] - db[i, i] * (cx - cy)

    return Corrected


def simulation_fixture(prismo, name, seed):
    """A reference ``Simulation`` with a dipole and a DFT ``FieldMonitor``."""
    from prismo import ElectricDipole, FieldMonitor, Simulation

    sim = Simulation(size=(1.2e-6, 0.9e-6, 0.0), resolution=2.5e7, pml_layers=3, courant_factor=0.5)
    src = ElectricDipole(position=(0.4e-6, 0.5e-6, 0.0), polarization="z", frequency=193e12,
                         pulse=True, pulse_width=2e-15)
    mon = FieldMonitor(center=(0.7e-6, 0.45e-6, 0.0), size=(0.0, 0.6e-6, 0.0), components=["Ez", "Hx", "Hy"],
                       time_domain=True, frequencies=[1.8e14, 1.93e14, 2.1e14])
    sim.add_source(src)
    sim.add_monitor(mon)
    nsteps = 12
    for _ in range(nsteps):
        sim.step()
    arrays = {f"out_{c}": np.asarray(sim.fields[c]) for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
    for c in ("Ez", "Hx", "Hy"):
        arrays[f"dft_{c}"] = np.stack([mon.get_frequency_data(c, f) for f in mon.frequencies])
        arrays[f"td_{c}"] = mon.get_time_data(c)[1]
    src_index = [list(map(int, np.asarray(ix).ravel())) for ix in src._source_region["Ez"]]
    mon_index = {c: [list(map(int, np.asarray(ix).ravel())) for ix in mon._monitor_region[c]]
                 for c in ("Ez", "Hx", "Hy")}
    arrays["meta"] = np.array(json.dumps({
        "size": [1.2e-6, 0.9e-6, 0.0], "resolution": 2.5e7, "layers": 3, "courant": 0.5,
        "nsteps": nsteps, "dt": sim.dt, "time": sim.current_time, "dims": sim.grid.dimensions,
        "src": {"position": [0.4e-6, 0.5e-6, 0.0], "frequency": 193e12, "pulse_width": 2e-15},
        "mon": {"center": [0.7e-6, 0.45e-6, 0.0], "size": [0.0, 0.6e-6, 0.0],
                "frequencies": [1.8e14, 1.93e14, 2.1e14]},
        "src_index_Ez": src_index, "mon_index": mon_index,
    }))
    save(name, **arrays)


def scalar_fixture(prismo, name):
    """CPML profiles, ADE coefficients, waveforms, grid semantics."""
    from prismo import CPML, DebyeMaterial, DrudeMaterial, LorentzMaterial, PMLParams
    from prismo.core.grid import GridSpec, YeeGrid
    from prismo.materials.dispersion import LorentzPole
    from prismo.sources.waveform import ContinuousWave, GaussianPulse

    out = {}
    g3 = YeeGrid(GridSpec(size=(1.0e-6, 0.8e-6, 0.6e-6), resolution=5e7, boundary_layers=8))
    cp = CPML(g3, PMLParams(thickness=8))
    out["cpml_dims"] = np.array(g3.dimensions)
    out["cpml_dt"] = np.array(g3.suggest_time_step(safety_factor=0.9))
    out["cpml_dmax"] = np.array(max(g3.spacing))
    for ax in ("x", "y", "z"):
        out[f"cpml_b{ax}"] = np.asarray(getattr(cp, f"b{ax}"))
        out[f"cpml_a{ax}"] = np.asarray(getattr(cp, f"a{ax}"))
    out["cpml_kappa"] = np.asarray(cp.kappa_pml)
    out["cpml_sigma"] = np.asarray(cp.sigma_pml)
    dt = 1.9e-17
    out["ade_dt"] = np.array(dt)
    lor = LorentzMaterial(1.5, [LorentzPole(omega_0=4e15, gamma=2e14, delta_epsilon=1.2),
                                LorentzPole(omega_0=5.5e15, gamma=4e14, delta_epsilon=0.7)])
    lc = lor.get_ade_coefficients(dt)
    out["lorentz"] = np.array([[p["C0"], p["C1"], p["C2"], p["C3"]] for p in lc["poles"]])
    out["lorentz_params"] = np.array([[4e15, 2e14, 1.2], [5.5e15, 4e14, 0.7]])
    dc = DrudeMaterial(1.0, 1.37e16, 1.0e14).get_ade_coefficients(dt)
    out["drude"] = np.array([dc["C0"], dc["C1"]])
    bc = DebyeMaterial(2.0, 5.0, 3e-15).get_ade_coefficients(dt)
    out["debye"] = np.array([bc["C0"], bc["C1"]])
    w = np.linspace(1.0e15, 2.0e15, 7)
    out["eps_w"] = w
    out["eps_lorentz"] = lor.permittivity(w)
    out["eps_drude"] = DrudeMaterial(1.0, 1.37e16, 1.0e14).permittivity(w)
    ts = np.linspace(0.0, 80e-15, 41)
    gp = GaussianPulse(frequency=193e12, pulse_width=10e-15, amplitude=1.3, phase=0.2)
    out["wave_t"] = ts
    out["wave_gauss"] = np.array([gp(t) for t in ts])
    out["wave_cw"] = np.array([ContinuousWave(frequency=193e12, amplitude=0.7, phase=0.1)(t) for t in ts])
    # grid semantics
    recs = []
    for size, res, layers in [((10e-6, 5e-6, 0.0), 50e6, 20), ((1.0e-6, 0.8e-6, 0.6e-6), 5e7, 8),
                              ((9.19e-6, 4.19e-6, 0.0), 5e7, 20)]:
        g = YeeGrid(GridSpec(size=size, resolution=res, boundary_layers=layers))
        r = {"size": size, "res": res, "layers": layers, "dims": g.dimensions,
             "shapes": {c: g.get_field_shape(c) for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")},
             "dt05": g.suggest_time_step(0.5), "courant": g.get_courant_number(g.suggest_time_step(0.5)),
             "p2i": [g.point_to_index(p) for p in [(0.0, 0.0, 0.0), (size[0] / 2, size[1] / 2, size[2] / 2),
                                                   (size[0], size[1], size[2]), (-1e-6, 3e-6, 0.1e-6)]],
             "idx": {c: [list(map(int, np.asarray(ix).ravel())) for ix in
                         g.get_component_indices(c, 3, 9, 2, 5, 1, 4)] for c in ("Ex", "Ez", "Hy")}}
        recs.append(r)
    out["grids"] = np.array(json.dumps(recs))
    save(name, **out)


def main():
    if len(sys.argv) < 2:
        raise SystemExit("usage: make_golden.py REFERENCE_CHECKOUT")
    root = sys.argv[1]
    prismo = import_reference(root)
    stepper_fixture(prismo, "ref_l0_3d.npz", (0.9e-6, 0.7e-6, 0.6e-6), 1e7, 2, 10, seed=1, lossy=True)
    stepper_fixture(prismo, "ref_l0_2d.npz", (1.7e-6, 1.3e-6, 0.0), 1e7, 3, 12, seed=2, lossy=True)
    stepper_fixture(prismo, "ref_l1_3d.npz", (0.9e-6, 0.7e-6, 0.6e-6), 1e7, 2, 30, seed=3, lossy=True,
                    corrected=True)
    stepper_fixture(prismo, "ref_l1_2d.npz", (1.7e-6, 1.3e-6, 0.0), 1e7, 3, 40, seed=4, lossy=True,
                    corrected=True)
    simulation_fixture(prismo, "ref_sim_2d.npz", seed=5)
    scalar_fixture(prismo, "ref_scalars.npz")


if __name__ == "__main__":
    main()
