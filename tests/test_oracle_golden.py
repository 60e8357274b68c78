"""Pin the CPU oracle against fixtures produced by running the reference itself
(tests/golden/make_golden.py).  CPU only."""

import json
import os

import numpy as np
import pytest

from oracle import fdtd64 as O

COMPS = O.COMPONENTS


def load(golden_dir, name):
    z = np.load(os.path.join(golden_dir, name))
    meta = json.loads(str(z["meta"]))
    return z, meta


def run_stepper(z, meta, legacy):
    g = O.OracleGrid(tuple(meta["size"]), meta["resolution"], meta["layers"])
    assert list(g.dims) == list(meta["dims"])
    mats = {k: z[k] for k in ("eps_rel", "mu_rel", "sigma_e", "sigma_m")}
    o = O.OracleFDTD(g, meta["dt"], mats, legacy=legacy)
    for c in COMPS:
        o.F[c][...] = z[f"init_{c}"]
    o.run(meta["nsteps"])
    return o


@pytest.mark.parametrize("name", ["ref_l0_3d.npz", "ref_l0_2d.npz"])
def test_l0_matches_unmodified_reference_bitwise(golden_dir, name):
    z, meta = load(golden_dir, name)
    o = run_stepper(z, meta, legacy=True)
    for c in COMPS:
        np.testing.assert_array_equal(o.F[c], z[f"out_{c}"], err_msg=c)


@pytest.mark.parametrize("name", ["ref_l1_3d.npz", "ref_l1_2d.npz"])
def test_l1_matches_reference_with_index_fix(golden_dir, name):
    z, meta = load(golden_dir, name)
    o = run_stepper(z, meta, legacy=False)
    for c in COMPS:
        ref = z[f"out_{c}"]
        np.testing.assert_allclose(o.F[c], ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max(), err_msg=c)


def test_simulation_sources_and_dft(golden_dir):
    """Simulation.step ordering, dipole source indices, FieldMonitor DFT."""
    z, meta = load(golden_dir, "ref_sim_2d.npz")
    g = O.OracleGrid(tuple(meta["size"]), meta["resolution"], meta["layers"])
    assert list(g.dims) == list(meta["dims"])
    dt = g.suggest_dt(meta["courant"])
    assert dt == meta["dt"]
    o = O.OracleFDTD(g, dt, legacy=True)
    s = meta["src"]
    x0, x1, y0, y1, z0, z1 = g.region_bounds(s["position"], (0, 0, 0))
    idx = g.component_indices("Ez", x0, x1, y0, y1, z0, z1)
    assert [list(map(int, np.ravel(i))) for i in idx] == meta["src_index_Ez"]
    o.add_source("Ez", idx, O.gaussian_pulse(s["frequency"], s["pulse_width"]))
    m = meta["mon"]
    b = g.region_bounds(m["center"], m["size"])
    ids = {}
    for c in ("Ez", "Hx", "Hy"):
        ix = g.component_indices(c, *b)
        assert [list(map(int, np.ravel(i))) for i in ix] == meta["mon_index"][c]
        ids[c] = o.add_dft(c, ix, m["frequencies"])
    o.run(meta["nsteps"])
    assert o.time == meta["time"]
    for c in COMPS:
        np.testing.assert_array_equal(o.F[c], z[f"out_{c}"], err_msg=c)
    for c in ("Ez", "Hx", "Hy"):
        np.testing.assert_array_equal(o.dfts[ids[c]].data, z[f"dft_{c}"], err_msg=c)


def test_cpml_profile_matches_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "ref_scalars.npz"))
    dims = z["cpml_dims"]
    for ax, n in zip("xyz", dims):
        b, a, k = O.cpml_profile(int(n), 8, float(z["cpml_dmax"]), float(z["cpml_dt"]), eps0_scaled=False)
        np.testing.assert_allclose(b, z[f"cpml_b{ax}"], rtol=1e-15)
        np.testing.assert_allclose(a, z[f"cpml_a{ax}"], rtol=1e-15, atol=0)
    # kappa profile: pml.py:141-146; interior ones, graded edges
    _, _, k = O.cpml_profile(int(dims[0]), 8, float(z["cpml_dmax"]), float(z["cpml_dt"]))
    np.testing.assert_allclose(k[:8][::-1], z["cpml_kappa"], rtol=1e-15)


def test_ade_coefficients_match_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "ref_scalars.npz"))
    dt = float(z["ade_dt"])
    for row, (w0, g, de) in zip(z["lorentz"], z["lorentz_params"]):
        c = O.lorentz_coeffs(de, w0, g, dt)
        np.testing.assert_allclose([c["C0"], c["C1"], c["C2"], c["C3"]], row, rtol=1e-15)
    c = O.drude_coeffs(1.37e16, 1.0e14, dt)
    np.testing.assert_allclose([c["C0"], c["C1"]], z["drude"], rtol=1e-15)
    c = O.debye_coeffs(5.0, 2.0, 3e-15, dt)
    np.testing.assert_allclose([c["C0"], c["C1"]], z["debye"], rtol=1e-15)


def test_waveforms_match_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "ref_scalars.npz"))
    f = O.gaussian_pulse(193e12, 10e-15, amplitude=1.3, phase=0.2)
    np.testing.assert_array_equal([f(t) for t in z["wave_t"]], z["wave_gauss"])
    f = O.continuous_wave(193e12, amplitude=0.7, phase=0.1)
    np.testing.assert_array_equal([f(t) for t in z["wave_t"]], z["wave_cw"])


def test_grid_semantics_match_reference(golden_dir):
    z = np.load(os.path.join(golden_dir, "ref_scalars.npz"))
    for r in json.loads(str(z["grids"])):
        g = O.OracleGrid(tuple(r["size"]), r["res"], r["layers"])
        assert list(g.dims) == r["dims"]
        for c, s in r["shapes"].items():
            assert list(g.shape(c)) == s
        assert g.suggest_dt(0.5) == r["dt05"]
        assert g.courant(g.suggest_dt(0.5)) == r["courant"]
        size = r["size"]
        pts = [(0.0, 0.0, 0.0), (size[0] / 2, size[1] / 2, size[2] / 2), (size[0], size[1], size[2]),
               (-1e-6, 3e-6, 0.1e-6)]
        assert [list(g.point_to_index(p)) for p in pts] == r["p2i"]
        for c, want in r["idx"].items():
            got = [list(map(int, np.ravel(i))) for i in g.component_indices(c, 3, 9, 2, 5, 1, 4)]
            assert got == want


def test_oracle_tfsf_keeps_scattered_region_dark():
    """In vacuum with nothing to scatter, the scattered-field side of the TFSF plane
    stays dark at the centre of the cross-section while the total-field side carries
    the incident pulse; what reaches the scattered side is diffraction from the
    plane's transverse edges (the plane spans the whole cross-section)."""
    g = O.OracleGrid.from_total(48, 48, 72, 20e-9, 8)
    dt = g.suggest_dt(0.5)
    wf = O.gaussian_pulse(193e12, 1e-15)
    o = O.OracleFDTD(g, dt, cpml_layers=8, tfsf=O.TFSFPlane(k0=54, direction=-1, polarization="x", waveform=wf))
    tf = sf = 0.0
    for _ in range(230):
        o.step()
        col = o.F["Ex"][24, 23, :]
        tf = max(tf, np.abs(col[30:52]).max())
        sf = max(sf, np.abs(col[56:63]).max())
    assert tf > 0.3
    assert sf < 1e-2 * tf
