"""The reference-facing API (Simulation, FDTDSolver, MaxwellUpdater, sources,
monitors, backend) on the GPU, read like the reference's own tests."""

import json
import os

import numpy as np
import pytest

from oracle import fdtd64 as O

pytestmark = pytest.mark.gpu

COMPS = O.COMPONENTS


@pytest.fixture(scope="module")
def pg():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import prismo_gb300

    prismo_gb300.set_backend("cuda")
    return prismo_gb300


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def test_reference_simulation_fixture_through_the_api(pg, golden_dir):
    """The reference Simulation with an ElectricDipole and a DFT FieldMonitor
    (tests/golden/ref_sim_2d.npz), reproduced with the float64 reference stepper."""
    z = np.load(os.path.join(golden_dir, "ref_sim_2d.npz"))
    meta = json.loads(str(z["meta"]))
    sim = pg.Simulation(size=tuple(meta["size"]), resolution=meta["resolution"], pml_layers=meta["layers"],
                        courant_factor=meta["courant"], precision="fp64", mode="legacy")
    assert sim.dt == meta["dt"]
    s = meta["src"]
    sim.add_source(pg.ElectricDipole(position=tuple(s["position"]), polarization="z", frequency=s["frequency"],
                                     pulse=True, pulse_width=s["pulse_width"]))
    m = meta["mon"]
    mon = pg.FieldMonitor(center=tuple(m["center"]), size=tuple(m["size"]), components=["Ez", "Hx", "Hy"],
                          time_domain=True, frequencies=m["frequencies"])
    sim.add_monitor(mon)
    for _ in range(meta["nsteps"]):
        sim.step()
    assert sim.current_time == meta["time"]
    for c in COMPS:
        np.testing.assert_array_equal(sim.fields[c].to_numpy(), z[f"out_{c}"], err_msg=c)
    for c in ("Ez", "Hx", "Hy"):
        np.testing.assert_array_equal(mon.get_time_data(c)[1], z[f"td_{c}"], err_msg=c)
        got = np.stack([mon.get_frequency_data(c, f) for f in m["frequencies"]])
        assert rel(got, z[f"dft_{c}"]) <= 1e-6, (c, rel(got, z[f"dft_{c}"]))


def test_corrected_simulation_matches_oracle(pg):
    size = ((60 - 8 - 0.5) * 20e-9, (50 - 8 - 0.5) * 20e-9, 0.0)
    sim = pg.Simulation(size=size, resolution=1 / 20e-9, pml_layers=4, courant_factor=0.5)
    src = pg.ElectricDipole(position=(0.3e-6, 0.4e-6, 0.0), polarization="z", frequency=193e12, pulse_width=4e-15)
    sim.add_source(src)
    mon = pg.FieldMonitor(center=(0.6e-6, 0.4e-6, 0.0), size=(0.0, 0.5e-6, 0.0), components=["Ez"],
                          time_domain=False, frequencies=[180e12, 193e12, 210e12])
    sim.add_monitor(mon)
    sim.run(250 * sim.dt * (1 - 1e-12))
    assert sim.step_count == 250
    g = O.OracleGrid(size, 1 / 20e-9, 4)
    o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=4)
    o.add_source("Ez", src._source_region["Ez"], O.gaussian_pulse(193e12, 4e-15))
    d = o.add_dft("Ez", mon._monitor_region["Ez"], mon.frequencies)
    o.run(250)
    for c in COMPS:
        assert rel(sim.fields[c].to_numpy(), o.F[c]) <= 1e-5, c
    for i, f in enumerate(mon.frequencies):
        assert rel(mon.get_frequency_data("Ez", f), o.dfts[d].data[i]) <= 1e-4
    assert sim.check() == 0


def test_solver_run_steps_and_reference_coefficients(pg):
    grid = pg.YeeGrid(pg.GridSpec(size=(1.0e-6, 1.0e-6, 1.0e-6), resolution=3e7, boundary_layers=3))
    dt = grid.suggest_time_step(safety_factor=0.5)
    up = pg.MaxwellUpdater(grid, dt)
    # tests/test_core_solver.py:140-153 (vacuum coefficients)
    assert np.allclose(up.Ca.to_numpy(), 1.0)
    assert np.allclose(up.Cb.to_numpy(), dt / up.eps0)
    assert np.allclose(up.Da.to_numpy(), 1.0)
    assert np.allclose(up.Db.to_numpy(), dt / up.mu0)
    nx, ny, nz = grid.dimensions
    up2 = pg.MaxwellUpdater(grid, dt, {"eps_rel": np.full((nx, ny, nz), 11.9)})
    assert np.allclose(up2.Cb.to_numpy(), dt / (up2.eps0 * 11.9))
    with pytest.raises(ValueError):
        pg.MaxwellUpdater(grid, grid.suggest_time_step(1.2))
    solver = pg.FDTDSolver(grid, dt, pml=3)
    solver.fields["Ez"][nx // 2, ny // 2, nz // 2] = 1.0
    solver.run_steps(30)
    assert solver.step_count == 30
    og = O.OracleGrid((1.0e-6, 1.0e-6, 1.0e-6), 3e7, 3)
    o = O.OracleFDTD(og, dt, cpml_layers=3)
    o.F["Ez"][nx // 2, ny // 2, nz // 2] = 1.0
    o.run(30)
    # Hz stays zero by symmetry for an Ez excitation: compare against the norm of
    # the whole E or H family instead of each component's own norm
    for fam in ("E", "H"):
        cs = [c for c in COMPS if c[0] == fam]
        scale = np.sqrt(sum(np.linalg.norm(o.F[c]) ** 2 for c in cs))
        for c in cs:
            assert np.linalg.norm(solver.fields[c].to_numpy() - o.F[c]) / scale <= 1e-5, c
    info = solver.get_simulation_info()
    assert info["step_count"] == 30 and info["field_energy"] > 0
    solver.reset()
    assert float(np.max(np.abs(solver.fields["Ez"]))) == 0.0


def test_backend_arrays_stay_on_device(pg):
    b = pg.get_backend()
    assert b.name == "cuda" and b.is_gpu
    a = b.asarray(np.arange(12.0).reshape(3, 4))
    assert a.tensor.is_cuda
    assert b.sum(a) == 66.0
    assert b.max(a) == 11.0
    np.testing.assert_allclose(b.to_numpy(b.sqrt(a)), np.sqrt(np.arange(12.0).reshape(3, 4)))
    a[np.ix_([0, 2], [1, 3])] += 1.0
    assert b.to_numpy(a)[2, 3] == 12.0
    assert np.max(np.abs(a)) == 12.0
    with pytest.raises(ValueError):
        pg.set_backend("metal")
    pg.set_backend("cuda")


def test_tfsf_through_simulation(pg):
    n = 36
    size = ((24 - 8 - 0.5) * 20e-9, (22 - 8 - 0.5) * 20e-9, (60 - 8 - 0.5) * 20e-9)
    sim = pg.Simulation(size=size, resolution=1 / 20e-9, pml_layers=4, courant_factor=0.5)
    src = pg.TFSFSource(center=(0.1e-6, 0.1e-6, 0.5e-6), size=(0, 0, 0), direction="-z", polarization="x",
                        frequency=193e12, pulse_width=3e-15)
    sim.add_source(src)
    k0 = src.plane_index()
    for _ in range(n):
        sim.step()
    g = O.OracleGrid(size, 1 / 20e-9, 4)
    o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=4,
                     tfsf=O.TFSFPlane(k0=k0, direction=-1, polarization="x", waveform=O.gaussian_pulse(193e12, 3e-15)))
    o.run(n)
    for c in COMPS:
        assert rel(sim.fields[c].to_numpy(), o.F[c]) <= 1e-5, c


def test_beam_and_mode_sources_through_simulation(pg):
    """GaussianBeamSource (E and H/377 soft sources over a beam profile) and
    ModeSource (mode profiles times A w(t) cos(phase - omega t)) through the
    Simulation API on the device, against the float64 oracle with the same
    injections: each component's L2 error <= 1e-5 of its field family's norm."""
    size = ((40 - 8 - 0.5) * 20e-9, (36 - 8 - 0.5) * 20e-9, (32 - 8 - 0.5) * 20e-9)
    sim = pg.Simulation(size=size, resolution=1 / 20e-9, pml_layers=4, courant_factor=0.5)
    gb = pg.GaussianBeamSource(center=(0.2e-6, 0.28e-6, 0.24e-6), size=(0.0, 0.2e-6, 0.16e-6), direction="x",
                               polarization="z", frequency=193e12, beam_waist=0.08e-6, pulse_width=4e-15)
    sim.add_source(gb)
    mc, msz = (0.45e-6, 0.25e-6, 0.22e-6), (0.0, 0.12e-6, 0.1e-6)
    probe = pg.ModeSource(mc, msz, {}, "-x", pg.GaussianPulse(193e12, 4e-15), 193e12)
    probe.initialize(sim.grid)
    rng = np.random.default_rng(5)
    prof = {c: rng.standard_normal(int(np.prod([np.asarray(i).size for i in probe._source_region[c]])))
            for c in ("Ey", "Ez", "Hx")}
    ms = pg.ModeSource(mc, msz, prof, "-x", pg.GaussianPulse(193e12, 4e-15), 193e12, amplitude=0.7, phase=0.4)
    sim.add_source(ms)
    n = 120
    sim.run(n * sim.dt * (1 - 1e-12))
    assert sim.step_count == n
    g = O.OracleGrid(size, 1 / 20e-9, 4)
    o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=4)
    wf = O.gaussian_pulse(193e12, 4e-15)
    for comp, idx, w, fn in gb.injections():
        o.add_source(comp, idx, (lambda t, fn=fn: fn(wf(t))), weight=w)
    om = 2 * np.pi * 193e12
    for comp, idx, w, fn in ms.injections():
        o.add_source(comp, idx, (lambda t: 0.7 * wf(t) * np.cos(0.4 - om * t)), weight=w)
    o.run(n)
    # per component, relative to its family (components only excited indirectly are
    # small, so their own float32 relative error is not the measure)
    fam = {f: np.sqrt(sum(np.linalg.norm(o.F[c]) ** 2 for c in COMPS if c[0] == f)) for f in "EH"}
    for c in COMPS:
        assert np.abs(o.F[c]).max() > 0, c
        err = np.linalg.norm(sim.fields[c].to_numpy() - o.F[c]) / fam[c[0]]
        assert err <= 1e-5, (c, err)
    assert sim.check() == 0
