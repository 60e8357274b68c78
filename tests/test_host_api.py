"""Host-side logic of the package on CPU (no GPU): grid semantics, CPML profiles,
source amplitude tables, backend registry."""

import json
import os

import numpy as np
import pytest

from helpers import SOURCE_TREES
from oracle import fdtd64 as O


def test_grid_mirror_matches_reference_fixture(golden_dir):
    from prismo_gb300.grid import GridSpec, YeeGrid

    z = np.load(os.path.join(golden_dir, "ref_scalars.npz"))
    for r in json.loads(str(z["grids"])):
        g = YeeGrid(GridSpec(size=tuple(r["size"]), resolution=r["res"], boundary_layers=r["layers"]))
        assert list(g.dimensions) == r["dims"]
        for c, s in r["shapes"].items():
            assert list(g.get_field_shape(c)) == s
        assert g.suggest_time_step(0.5) == r["dt05"]
        size = r["size"]
        pts = [(0.0, 0.0, 0.0), (size[0] / 2, size[1] / 2, size[2] / 2), (size[0], size[1], size[2]),
               (-1e-6, 3e-6, 0.1e-6)]
        assert [list(g.point_to_index(p)) for p in pts] == r["p2i"]
        for c, want in r["idx"].items():
            got = [list(map(int, np.ravel(i))) for i in g.get_component_indices(c, 3, 9, 2, 5, 1, 4)]
            assert got == want


def test_cpml_coefficients_match_oracle():
    from prismo_gb300.pml import PMLParams, cpml_axis_coefficients

    for n, t in [(64, 8), (256, 12), (30, 3)]:
        b, a, k = cpml_axis_coefficients(n, PMLParams(thickness=t), 20e-9, 1.9e-17)
        b2, a2, k2 = O.cpml_profile(n, t, 20e-9, 1.9e-17)
        np.testing.assert_allclose(b, b2, rtol=1e-15)
        np.testing.assert_allclose(a, a2, rtol=1e-15, atol=0)
        np.testing.assert_allclose(k, k2, rtol=1e-15)


def test_source_amplitudes_follow_reference_expressions():
    from prismo_gb300.grid import YeeGrid
    from prismo_gb300.sources import ElectricDipole, PlaneWaveSource, amplitude_table

    g = YeeGrid.from_total((40, 30, 1), 20e-9, 5)
    d = ElectricDipole(position=(0.2e-6, 0.2e-6, 0.0), polarization="z", frequency=193e12, pulse_width=5e-15)
    pw = PlaneWaveSource(center=(0.2e-6, 0.2e-6, 0), size=(0, 0.3e-6, 0), direction="-x", polarization="z",
                         frequency=193e12, pulse_width=5e-15)
    for s in (d, pw):
        s.initialize(g)
    t = np.cumsum(np.full(50, 3e-17))
    tab = amplitude_table([d, pw], t)
    wf = O.gaussian_pulse(193e12, 5e-15)
    np.testing.assert_array_equal(tab[:, 0], [wf(x) for x in t])
    np.testing.assert_array_equal(tab[:, 1], [wf(x) * -1 for x in t])
    np.testing.assert_array_equal(tab[:, 2], [(wf(x) / 377.0) * -1 for x in t])


def test_backend_registry_without_gpu():
    import torch

    from prismo_gb300 import backend

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    assert backend.list_available_backends() == []
    with pytest.raises(ValueError):
        backend.set_backend("cuda")
    with pytest.raises(ValueError):
        backend.set_backend("numpy")


def test_materials_match_reference_coefficients(golden_dir):
    from prismo_gb300.materials import DebyeMaterial, DrudeMaterial, LorentzMaterial, LorentzPole

    z = np.load(os.path.join(golden_dir, "ref_scalars.npz"))
    dt = float(z["ade_dt"])
    lor = LorentzMaterial(1.5, [LorentzPole(omega_0=w0, gamma=g, delta_epsilon=de) for w0, g, de in z["lorentz_params"]])
    got = np.array([[p[k] for k in ("C0", "C1", "C2", "C3")] for p in lor.get_ade_coefficients(dt)["poles"]])
    np.testing.assert_allclose(got, z["lorentz"], rtol=1e-15)
    c = DrudeMaterial(1.0, 1.37e16, 1.0e14).get_ade_coefficients(dt)
    np.testing.assert_allclose([c["C0"], c["C1"]], z["drude"], rtol=1e-15)
    c = DebyeMaterial(2.0, 5.0, 3e-15).get_ade_coefficients(dt)
    np.testing.assert_allclose([c["C0"], c["C1"]], z["debye"], rtol=1e-15)
    np.testing.assert_allclose(lor.permittivity(z["eps_w"]), z["eps_lorentz"], rtol=1e-13)
    np.testing.assert_allclose(DrudeMaterial(1.0, 1.37e16, 1.0e14).permittivity(z["eps_w"]), z["eps_drude"],
                               rtol=1e-13)


def test_gaussian_beam_and_mode_sources_host_side():
    """GaussianBeamSource (sources/gaussian.py:167-298): E weights exp(-r^2/w0^2)
    over the region in C order, H the same with a / 377; ModeSource
    (sources/mode.py:198-361): A w(t) cos(phase - omega t), normal H signed."""
    from prismo_gb300.grid import YeeGrid
    from prismo_gb300.sources import GaussianBeamSource, GaussianPulse, ModeSource, amplitude_table

    g = YeeGrid.from_total((40, 30, 26), 20e-9, 4)
    gb = GaussianBeamSource(center=(0.3e-6, 0.2e-6, 0.18e-6), size=(0.0, 0.2e-6, 0.16e-6), direction="x",
                            polarization="z", frequency=193e12, beam_waist=0.1e-6, pulse_width=5e-15)
    gb.initialize(g)
    x0, x1, y0, y1, z0, z1 = gb._compute_source_region()
    ys, zs = np.meshgrid(np.arange(y0, y1), np.arange(z0, z1), indexing="ij")
    want = np.exp(-((g.index_to_coord(1, ys) - 0.2e-6) ** 2 + (g.index_to_coord(2, zs) - 0.18e-6) ** 2) / 1e-14)
    inj = gb.injections()
    assert [i[0] for i in inj] == ["Ez", "Hy"]
    np.testing.assert_allclose(inj[0][2].ravel(), want.ravel(), rtol=1e-14)
    np.testing.assert_allclose(inj[1][2].ravel(), want.ravel(), rtol=1e-14)
    t = np.cumsum(np.full(20, 3e-17))
    tab = amplitude_table([gb], t)
    wf = O.gaussian_pulse(193e12, 5e-15)
    np.testing.assert_array_equal(tab[:, 0], [wf(x) for x in t])
    np.testing.assert_array_equal(tab[:, 1], [wf(x) / 377.0 for x in t])

    ms_center, ms_size = (0.2e-6, 0.2e-6, 0.2e-6), (0.0, 0.1e-6, 0.1e-6)
    probe = ModeSource(ms_center, ms_size, {}, "-x", GaussianPulse(193e12, 5e-15), 193e12)
    probe.initialize(g)
    shp = {c: tuple(np.asarray(i).size for i in probe._source_region[c]) for c in ("Ey", "Ez", "Hx")}
    rng = np.random.default_rng(1)
    prof = {c: rng.standard_normal(int(np.prod(shp[c]))) for c in shp}
    ms = ModeSource(ms_center, ms_size, prof, "-x", GaussianPulse(193e12, 5e-15), 193e12, amplitude=2.0,
                    phase=0.3)
    ms.initialize(g)
    inj = {c: w for c, _, w, _ in ms.injections()}
    np.testing.assert_array_equal(inj["Ey"].ravel(), prof["Ey"])
    np.testing.assert_array_equal(inj["Hx"].ravel(), -prof["Hx"])  # -x: the normal H is negated
    a = amplitude_table([ms], t)[:, 0]
    np.testing.assert_allclose(a, 2.0 * np.array([wf(x) for x in t]) * np.cos(0.3 - 2 * np.pi * 193e12 * t),
                               rtol=1e-14, atol=1e-300)


def test_flux_monitor_interface_and_host_path():
    """FluxMonitor as the reference's tests construct it (tests/test_monitors_advanced.py
    TestFluxMonitor), and its host path (fields given on the host, no engine)
    against the flux.py:126-173 / 219-285 formulas evaluated directly."""
    from prismo_gb300 import FluxMonitor
    from prismo_gb300.grid import GridSpec, YeeGrid

    m = FluxMonitor(center=(0, 0, 0), size=(0, 1e-6, 0), direction="x", frequencies=[193e12])
    assert m.direction == "x" and m.frequencies is not None
    with pytest.raises(ValueError):
        FluxMonitor(center=(0, 0, 0), size=(0, 1e-6, 0), direction="w")
    grid = YeeGrid(GridSpec(size=(5e-6, 3e-6, 0), resolution=10e6))
    m = FluxMonitor(center=(0, 0, 0), size=(0, 1e-6, 0), direction="x")
    m.initialize(grid)
    assert m._power_flow_history == [] and m._time_history == []

    grid = YeeGrid(GridSpec(size=(1e-6, 0.8e-6, 0.6e-6), resolution=20e6))
    freqs = [180e12, 200e12]
    m = FluxMonitor(center=(0.5e-6, 0.4e-6, 0.3e-6), size=(0.5e-6, 0.0, 0.3e-6), direction="y", frequencies=freqs)
    m.initialize(grid)
    rng = np.random.default_rng(3)
    dt = 1e-17
    want = []
    dft = {c: 0 for c in m._TERMS["y"]}
    for n in range(5):
        fields = {c: rng.standard_normal(grid.get_field_shape(c)) for c in O.COMPONENTS}
        t = (n + 1) * dt
        m.update(fields, t, dt)
        a, b, c, d = (fields[k][m._plane[k]] for k in m._TERMS["y"])
        want.append(np.sum(a * b - c * d) * grid.dx * grid.dz)
        for k in m._TERMS["y"]:
            dft[k] = dft[k] + np.stack([fields[k][m._plane[k]] * np.exp(-2j * np.pi * f * t) * dt for f in freqs])
    t, p = m.get_time_domain_power()
    np.testing.assert_allclose(p, want, rtol=1e-12)
    np.testing.assert_allclose(t, dt * np.arange(1, 6))
    A, B, C, D = (dft[k] for k in m._TERMS["y"])
    spec = [0.5 * np.real(np.sum(A[i] * np.conj(B[i]) - C[i] * np.conj(D[i]))) * grid.dx * grid.dz
            for i in range(len(freqs))]
    np.testing.assert_allclose(m.get_frequency_domain_power(), spec, rtol=1e-12)
    assert m._plane["Ez"][1].ravel().size == 1  # a plane normal to y


def _reference_mode_matching():
    """utils/mode_matching.py of the reference when its source tree is present."""
    import importlib.util

    for root in SOURCE_TREES:
        p = os.path.join(root, "prismo", "utils", "mode_matching.py") if root else ""
        if p and os.path.exists(p):
            import sys
            import types

            # the module imports prismo.modes.solver.WaveguideMode for type hints only:
            # stand-ins while it loads, then the import table as it was
            names = ("prismo", "prismo.modes", "prismo.modes.solver")
            saved = {n: sys.modules.get(n) for n in names}
            try:
                for n in names:
                    sys.modules[n] = types.ModuleType(n)
                sys.modules["prismo.modes.solver"].WaveguideMode = object
                spec = importlib.util.spec_from_file_location("_ref_mode_matching", p)
                mod = importlib.util.module_from_spec(spec)
                spec.loader.exec_module(mod)
            finally:
                for n, m in saved.items():
                    if m is None:
                        sys.modules.pop(n, None)
                    else:
                        sys.modules[n] = m
            return mod
    return None


def test_mode_expansion_monitor_host_path_matches_reference_overlap():
    """ModeExpansionMonitor's per-step coefficients (host path) against the
    reference's own compute_mode_overlap (utils/mode_matching.py:41-131, unit
    spacing as mode_monitor.py:176-178 passes) on the same plane arrays, and its
    spectrum against the mode_monitor.py:171-175 accumulation."""
    from types import SimpleNamespace

    from prismo_gb300 import ModeExpansionMonitor
    from prismo_gb300.grid import GridSpec, YeeGrid

    mm = _reference_mode_matching()
    if mm is None:
        pytest.skip("reference source tree not present")
    grid = YeeGrid(GridSpec(size=(1e-6, 0.8e-6, 0.6e-6), resolution=20e6))
    rng = np.random.default_rng(5)
    mon = ModeExpansionMonitor(center=(0.5e-6, 0.4e-6, 0.3e-6), size=(0.0, 0.5e-6, 0.3e-6), modes=[],
                               direction="x", frequencies=[190e12, 200e12])
    mon.initialize(grid)
    shp = tuple(np.broadcast_shapes(*(a.shape for a in mon._plane["Ey"])))
    modes = [SimpleNamespace(**{c: rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
                                for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}) for _ in range(2)]
    mon = ModeExpansionMonitor(center=(0.5e-6, 0.4e-6, 0.3e-6), size=(0.0, 0.5e-6, 0.3e-6), modes=modes,
                               direction="x", frequencies=[190e12, 200e12])
    mon.initialize(grid)
    dt = 1e-17
    want = [[], []]
    for n in range(4):
        fields = {c: rng.standard_normal(grid.get_field_shape(c)) for c in O.COMPONENTS}
        mon.update(fields, (n + 1) * dt, dt)
        sim = {c: fields[c][mon._plane[c]] if c in mon._plane else np.zeros(shp)
               for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
        for m, mode in enumerate(modes):
            want[m].append(mm.compute_mode_overlap(sim["Ex"], sim["Ey"], sim["Ez"], sim["Hx"], sim["Hy"], sim["Hz"],
                                                   mode, direction="x", dx=1.0, dy=1.0))
    for m in range(2):
        np.testing.assert_allclose(mon.get_mode_coefficient(m), want[m], rtol=1e-12)
        t = dt * np.arange(1, 5)
        spec = [np.sum(np.array(want[m]) * np.exp(-1j * w * t) * dt) for w in mon.omega]
        np.testing.assert_allclose(mon.get_mode_coefficient(m, "frequency"), spec, rtol=1e-12)


def test_tensor_material_matches_reference_inverses():
    """prismo_gb300.tensor containers against the reference's TensorMaterial
    (materials/tensor.py:110-312): full matrices, diagonal test, inverses."""
    from prismo_gb300.tensor import TensorComponents, TensorMaterial
    from helpers import SOURCE_TREES, import_reference

    import_reference(SOURCE_TREES)
    from prismo.materials import tensor as RT

    rng = np.random.default_rng(2)
    cases = [dict(xx=2.0, yy=3.0, zz=4.0), dict(xx=2.2, yy=2.5, zz=3.1, xy=0.3, xz=-0.2, yz=0.1, yx=0.25),
             dict(xx=rng.uniform(2, 4, (3, 4)), yy=rng.uniform(2, 4, (3, 4)), zz=rng.uniform(2, 4, (3, 4)),
                  xy=rng.uniform(-0.3, 0.3, (3, 4)))]
    for kw in cases:
        ours = TensorMaterial(TensorComponents(**kw))
        ref = RT.TensorMaterial(RT.TensorComponents(**kw))
        assert ours.is_diagonal == ref.is_diagonal
        np.testing.assert_array_equal(ours.epsilon_tensor, np.asarray(ref.epsilon_tensor))
        np.testing.assert_allclose(ours.get_inverse_epsilon(), ref.get_inverse_epsilon(), rtol=1e-14, atol=1e-15)
        np.testing.assert_allclose(ours.get_inverse_mu(), ref.get_inverse_mu(), rtol=1e-14)


def test_mode_port_region_and_interpolation_match_reference():
    """ModePort's plane bounds and interpolated profiles against the reference's
    own ModePort (boundaries/mode_port.py:112-259) on the same grid and modes."""
    from prismo_gb300.grid import GridSpec, YeeGrid
    from prismo_gb300.ports import ModePort, ModePortConfig
    from helpers import SOURCE_TREES, import_reference

    import_reference(SOURCE_TREES)
    from prismo.boundaries import mode_port as RP
    from prismo.core.grid import GridSpec as RGridSpec
    from prismo.core.grid import YeeGrid as RYeeGrid
    from prismo.modes.solver import WaveguideMode

    rng = np.random.default_rng(4)
    from helpers import port_modes

    modes = port_modes(rng)
    rmodes = [WaveguideMode(**vars(m)) for m in modes]
    spec = dict(size=(1.2e-6, 1.0e-6, 0.8e-6), resolution=20e6)
    for direction, center, size in (("+x", (0.5e-6, 0.5e-6, 0.4e-6), (0.0, 0.6e-6, 0.5e-6)),
                                    ("-y", (0.6e-6, 0.45e-6, 0.4e-6), (0.7e-6, 0.0, 0.5e-6)),
                                    ("+z", (0.6e-6, 0.5e-6, 0.3e-6), (0.7e-6, 0.6e-6, 0.0))):
        ours = ModePort(ModePortConfig(center, size, direction, modes, inject=True))
        ours.initialize(YeeGrid(GridSpec(**spec)))
        ref = RP.ModePort(RP.ModePortConfig(center, size, direction, rmodes, inject=True))
        ref.initialize(RYeeGrid(RGridSpec(**spec)))
        assert ours._port_region == ref._port_region
        for a, b in zip(ours._interpolated_modes, ref._interpolated_modes):
            for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz"):
                np.testing.assert_array_equal(getattr(a, c), getattr(b, c))


def test_monitor_port_and_tensor_error_paths():
    """Errors the reference raises (monitors/flux.py:247-248, mode_monitor.py:63-64,
    246-256) and the device classes' own input checks, without a GPU."""
    from types import SimpleNamespace

    from prismo_gb300 import FluxMonitor, ModeExpansionMonitor
    from prismo_gb300.grid import GridSpec, YeeGrid
    from prismo_gb300.ports import ModePort, ModePortConfig

    grid = YeeGrid(GridSpec(size=(1e-6, 0.8e-6, 0.0), resolution=20e6))
    m = FluxMonitor(center=(0.5e-6, 0.4e-6, 0), size=(0, 0.4e-6, 0), direction="x")
    m.initialize(grid)
    with pytest.raises(RuntimeError):
        m.get_frequency_domain_power()
    assert m.get_transmission() == 0.0  # no steps yet: the reference returns 0.0
    with pytest.raises(ValueError):
        ModeExpansionMonitor(center=(0, 0, 0), size=(0, 1e-6, 0), modes=[], direction="q")
    mm = ModeExpansionMonitor(center=(0.5e-6, 0.4e-6, 0), size=(0, 0.4e-6, 0), modes=[])
    mm.initialize(grid)
    with pytest.raises(ValueError):
        mm.get_mode_coefficient(0, domain="space")
    with pytest.raises(RuntimeError):
        mm.get_mode_transmission(0)
    port = ModePort(ModePortConfig((0.5e-6, 0.4e-6, 0), (0, 0.4e-6, 0), "+x", []))
    with pytest.raises(ValueError):
        port.initialize(grid)  # mode ports index [x, y, z]: 3D grids only
    assert port.sign == 1 and port.axis == "x"
    assert ModePort(ModePortConfig((0, 0, 0), (0, 0, 0), "-z", [])).sign == -1


def test_anisotropic_updater_rejects_host_arrays():
    torch = pytest.importorskip("torch")
    from prismo_gb300.tensor import AnisotropicUpdater, TensorComponents, TensorMaterial

    up = AnisotropicUpdater(TensorMaterial(TensorComponents(xx=2.0, yy=2.0, zz=2.0)), 1e-17)
    x = [torch.zeros(4, 4, dtype=torch.float64) for _ in range(3)]
    with pytest.raises(TypeError):
        up.update_e_from_curl_h(x, x)


def test_dispersive_byte_models():
    """Algorithmic bytes per cell update of the 384x384x192 dispersive
    configuration (Drude + 2 Lorentz on the metal half, 12-cell CPML, two
    64-frequency planes): 60 B of fields and Cb, 32 B of psi on the slab fraction,
    24 + 2 x 48 B of ADE auxiliaries on the metal half, and the DFT either updated
    every step (32 B per frequency and plane point) or through the 16-step ring."""
    from prismo_gb300.workloads import config_3d_dispersive, dispersive_bytes_per_cell

    dims = (384, 384, 192)
    _, box, _, _ = config_3d_dispersive(dims, z_metal=96)
    n = 384 * 384 * 192
    base = 60 + 32 * (24 / 384 + 24 / 384 + 24 / 192) + 0.5 * (24 + 2 * 48)
    plane = 2 * 384 * 384 / n
    assert abs(dispersive_bytes_per_cell(dims, 12, box, 2, 2, 64) - (base + plane * 64 * 32)) < 1e-9
    assert abs(dispersive_bytes_per_cell(dims, 12, box, 2, 2, 64, "ring") - (base + plane * (64 * 2 + 8))) < 1e-9
    assert abs(dispersive_bytes_per_cell(dims, 12, box, 2, 2, 64) - 149.333) < 1e-3
