"""ModePort on device fields: injection against the reference's in-place NumPy
update (mode_port.py:327-365; float64 sum rounded once, so both precisions match
bit for bit) and extraction against utils/mode_matching.py:41-171 evaluated with
NumPy on the same plane (rel 1e-12 in float64, 1e-6 in float32).  The port's
plane and interpolated profiles are pinned to the reference in test_host_api.py."""

import numpy as np
import pytest

from helpers import port_modes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def pg():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import prismo_gb300

    prismo_gb300.set_backend("cuda")
    return prismo_gb300


def overlap(sim, mode, axis, dx, dy):
    """compute_mode_overlap / compute_mode_power of utils/mode_matching.py, restated."""
    t = {"x": ("Ey", "Hz", "Ez", "Hy"), "y": ("Ez", "Hx", "Ex", "Hz"), "z": ("Ex", "Hy", "Ey", "Hx")}[axis]
    m = {c: getattr(mode, c) for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}
    s_sim = sim[t[0]] * np.conj(m[t[1]]) - sim[t[2]] * np.conj(m[t[3]])
    s_mode = m[t[0]] * np.conj(sim[t[1]]) - m[t[2]] * np.conj(sim[t[3]])
    ov = 0.5 * np.sum(s_sim + s_mode) * dx * dy
    p = abs(0.5 * np.real(np.sum(m[t[0]] * np.conj(m[t[1]]) - m[t[2]] * np.conj(m[t[3]]))) * dx * dy)
    return complex(ov / p) if p > 1e-20 else 0.0


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_mode_port_inject_and_extract(pg, dtype):
    from prismo_gb300.grid import GridSpec, YeeGrid
    from prismo_gb300.ports import ModePort, ModePortConfig

    rng = np.random.default_rng(12)
    grid = YeeGrid(GridSpec(size=(1.2e-6, 1.0e-6, 0.8e-6), resolution=20e6))
    modes = port_modes(rng)
    for direction, center, size in (("+x", (0.5e-6, 0.5e-6, 0.4e-6), (0.0, 0.6e-6, 0.5e-6)),
                                    ("-y", (0.6e-6, 0.45e-6, 0.4e-6), (0.7e-6, 0.0, 0.5e-6)),
                                    ("+z", (0.6e-6, 0.5e-6, 0.3e-6), (0.7e-6, 0.6e-6, 0.0))):
        fields = pg.ElectromagneticFields(grid, dtype=dtype)
        host = {c: rng.standard_normal(grid.get_field_shape(c)).astype(dtype) for c in fields._fields}
        for c, v in host.items():
            fields[c] = v
        port = ModePort(ModePortConfig(center, size, direction, modes, inject=True))
        port.initialize(grid)
        t, dt, amps = 7.3e-15, 3.3e-17, [1.0, 0.4 - 0.3j]
        port.inject_fields(fields, t, dt, amps)
        idx = port._index()
        inj = {"x": ("Ey", "Ez", "Hx"), "y": ("Ex", "Ez", "Hy"), "z": ("Ex", "Ey", "Hz")}[port.axis]
        for mode, a in zip(port._interpolated_modes, amps):  # mode_port.py:291-305, 327-365
            ar = (a * np.exp(1j * (2 * np.pi * mode.frequency * t))).real
            for c in inj:
                host[c][idx] += ar * getattr(mode, c).real
        for c in host:
            np.testing.assert_array_equal(fields[c].to_numpy(), host[c], err_msg=(direction, c))
        got = port.extract_mode_coefficients(fields, t)
        sim = {c: host[c][idx].astype(np.float64) for c in host}
        dx, dy = port._spacing()
        want = [overlap(sim, m, port.axis, dx, dy) for m in port._interpolated_modes]
        tol = 1e-12 if dtype == np.float64 else 1e-6
        np.testing.assert_allclose(got, want, rtol=tol)
        assert port.get_time_points() == [t] and port.get_mode_coefficient(1) == [got[1]]
