"""FluxMonitor on the device (flux.cu) against the float64 oracle: the per-step
power through the plane (monitors/flux.py:126-173) and P(f) = 1/2 Re sum
(E x H*)_n dA from the DFTs (flux.py:219-285), with the oracle's fields taken at
the same plane indices.  Float32 fields against float64: the history agrees to
rel L2 <= 1e-4 over the run, the spectrum to <= 1e-4."""

import numpy as np
import pytest

from oracle import fdtd64 as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import prismo_gb300

    prismo_gb300.set_backend("cuda")
    return prismo_gb300


def rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300)


def oracle_flux(o, mon, freqs, nsteps):
    terms = mon._TERMS[mon.direction]
    ids = [o.add_dft(c, mon._plane[c], freqs) for c in terms]
    hist = []
    for _ in range(nsteps):
        o.step()
        a, b, c, d = (o.F[k][mon._plane[k]] for k in terms)
        hist.append(np.sum(a * b - c * d) * mon._dA)
    A, B, C, D = (o.dfts[i].data for i in ids)
    spec = [0.5 * np.real(np.sum(A[f] * np.conj(B[f]) - C[f] * np.conj(D[f]))) * mon._dA for f in range(len(freqs))]
    return np.array(hist), np.array(spec)


def test_flux_monitor_2d_matches_oracle(pg):
    size = ((60 - 8 - 0.5) * 20e-9, (50 - 8 - 0.5) * 20e-9, 0.0)
    sim = pg.Simulation(size=size, resolution=1 / 20e-9, pml_layers=4, courant_factor=0.5)
    src = pg.ElectricDipole(position=(0.3e-6, 0.4e-6, 0.0), polarization="z", frequency=193e12, pulse_width=4e-15)
    sim.add_source(src)
    freqs = [180e12, 193e12, 210e12]
    mon = pg.FluxMonitor(center=(0.6e-6, 0.4e-6, 0.0), size=(0.0, 0.5e-6, 0.0), direction="x", frequencies=freqs)
    sim.add_monitor(mon)
    n = 250
    sim.run(n * sim.dt * (1 - 1e-12))
    g = O.OracleGrid(size, 1 / 20e-9, 4)
    o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=4)
    o.add_source("Ez", src._source_region["Ez"], O.gaussian_pulse(193e12, 4e-15))
    hist, spec = oracle_flux(o, mon, freqs, n)
    t, p = mon.get_time_domain_power()
    assert p.shape == (n,) and np.abs(hist).max() > 0
    assert rel(p, hist) <= 1e-4, rel(p, hist)
    np.testing.assert_allclose(t, sim.dt * np.arange(1, n + 1), rtol=1e-12)
    P = mon.get_frequency_domain_power()
    assert rel(P, spec) <= 1e-4, (P, spec)
    assert mon.get_frequency_domain_power(1) == pytest.approx(P[1])
    np.testing.assert_allclose(mon.get_transmission(reference_power=P), 1.0)
    assert sim.check() == 0


def test_flux_monitor_3d_fused_matches_oracle(pg):
    """3D (fused stepper, graph-replayed time loop): flux through a z plane."""
    size = ((40 - 6 - 0.5) * 20e-9, (36 - 6 - 0.5) * 20e-9, (44 - 6 - 0.5) * 20e-9)
    sim = pg.Simulation(size=size, resolution=1 / 20e-9, pml_layers=3, courant_factor=0.5)
    src = pg.ElectricDipole(position=(0.3e-6, 0.3e-6, 0.25e-6), polarization="x", frequency=193e12,
                            pulse_width=3e-15)
    sim.add_source(src)
    freqs = [185e12, 200e12]
    mon = pg.FluxMonitor(center=(0.3e-6, 0.3e-6, 0.5e-6), size=(0.4e-6, 0.4e-6, 0.0), direction="z",
                         frequencies=freqs)
    sim.add_monitor(mon)
    n = 160
    sim.run(n * sim.dt * (1 - 1e-12))
    g = O.OracleGrid(size, 1 / 20e-9, 3)
    o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=3)
    o.add_source("Ex", src._source_region["Ex"], O.gaussian_pulse(193e12, 3e-15))
    hist, spec = oracle_flux(o, mon, freqs, n)
    _, p = mon.get_time_domain_power()
    assert np.abs(hist).max() > 0
    assert rel(p, hist) <= 1e-4, rel(p, hist)
    assert rel(mon.get_frequency_domain_power(), spec) <= 1e-4
    assert sim.check() == 0


def test_mode_expansion_monitor_matches_oracle(pg):
    """ModeExpansionMonitor on the device: per-step coefficients and spectra of two
    modes on a 2D x plane against the same weights (pinned to the reference's
    compute_mode_overlap in test_host_api.py) applied to the oracle's fields."""
    from types import SimpleNamespace

    size = ((60 - 8 - 0.5) * 20e-9, (50 - 8 - 0.5) * 20e-9, 0.0)
    sim = pg.Simulation(size=size, resolution=1 / 20e-9, pml_layers=4, courant_factor=0.5)
    src = pg.ElectricDipole(position=(0.3e-6, 0.4e-6, 0.0), polarization="z", frequency=193e12, pulse_width=4e-15)
    sim.add_source(src)
    rng = np.random.default_rng(7)
    probe = pg.ModeExpansionMonitor(center=(0.6e-6, 0.4e-6, 0.0), size=(0.0, 0.5e-6, 0.0), modes=[])
    probe.initialize(sim.grid)
    npts = probe._plane["Ez"][1].size
    y = np.linspace(-1, 1, 2 * npts + 3)  # another length: resized to the plane as the reference does
    modes = [SimpleNamespace(Ex=0 * y, Ey=0 * y, Ez=np.exp(-4 * y**2) * (1 + 0.3j * k), Hx=0 * y,
                             Hy=-np.exp(-4 * y**2) / 377.0 * (1 - 0.2j * k), Hz=0 * y) for k in range(2)]
    freqs = [185e12, 193e12, 205e12]
    mon = pg.ModeExpansionMonitor(center=(0.6e-6, 0.4e-6, 0.0), size=(0.0, 0.5e-6, 0.0), modes=modes,
                                  direction="x", frequencies=freqs)
    sim.add_monitor(mon)
    n = 250
    sim.run(n * sim.dt * (1 - 1e-12))
    g = O.OracleGrid(size, 1 / 20e-9, 4)
    o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=4)
    o.add_source("Ez", src._source_region["Ez"], O.gaussian_pulse(193e12, 4e-15))
    terms = mon._TERMS["x"]
    want = []
    for _ in range(n):
        o.step()
        vals = [o.F[c][mon._plane[c]] for c in terms]
        want.append([sum(np.sum(mon._weights[m, q] * vals[q]) for q in range(4)) for m in range(2)])
    want = np.array(want)
    t = sim.dt * np.arange(1, n + 1)
    for m in range(2):
        got = np.array(mon.get_mode_coefficient(m))
        assert np.abs(want[:, m]).max() > 0
        assert rel(got, want[:, m]) <= 1e-4, rel(got, want[:, m])
        spec = [np.sum(want[:, m] * np.exp(-2j * np.pi * f * t)) * sim.dt for f in freqs]
        assert rel(mon.get_mode_coefficient(m, "frequency"), spec) <= 1e-4
    assert mon.get_mode_power(0, 1) == pytest.approx(abs(mon.get_mode_coefficient(0, "frequency")[1]) ** 2)
    assert set(mon.compute_s_parameters()) == {"S_11", "S_21"}
    assert sim.check() == 0
