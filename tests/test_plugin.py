"""The plugin inside the reference package (CPU part: registration must not
disturb the reference's own NumPy path; GPU part runs the reference API with the
cuda backend when a GPU is present).  The reference is imported from its source
tree (the harness shim of tests/golden/make_golden.py); skipped when absent."""

import os

import numpy as np
import pytest

from helpers import INSTALLED, SOURCE_TREES  # noqa: F401
from helpers import import_reference as _import_reference


def _registered(candidates):
    p = _import_reference(candidates)
    from prismo_gb300 import plugin

    plugin.register(p)
    return p


@pytest.fixture(scope="module")
def prismo():
    return _registered([INSTALLED] + SOURCE_TREES)


@pytest.fixture(scope="module")
def prismo_installed():
    return _registered([INSTALLED])


def test_registration_keeps_numpy_path(prismo):
    prismo.set_backend("numpy")
    assert "numpy" in prismo.list_available_backends()
    from prismo.core.grid import GridSpec, YeeGrid
    from prismo.core.solver import MaxwellUpdater

    grid = YeeGrid(GridSpec(size=(1.0e-6, 1.0e-6, 0.0), resolution=1e7))
    dt = grid.suggest_time_step(0.5)
    up = MaxwellUpdater(grid, dt)
    assert type(up).__module__ == "prismo.core.solver"
    assert np.allclose(up.Cb, dt / up.eps0)


def test_cuda_selection_follows_device_availability(prismo):
    import torch

    if torch.cuda.is_available():
        assert "cuda" in prismo.list_available_backends()
    else:
        assert "cuda" not in prismo.list_available_backends()
        with pytest.raises(ValueError):
            prismo.set_backend("cuda")
    with pytest.raises(ValueError):
        prismo.set_backend("no-such-backend")
    prismo.set_backend("numpy")


@pytest.mark.gpu
def test_reference_api_on_cuda(prismo_installed):
    prismo = prismo_installed
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import fdtd64 as O

    prismo.set_backend("cuda")
    try:
        from prismo import ElectricDipole, FieldMonitor, Simulation

        size = ((60 - 8 - 0.5) * 20e-9, (50 - 8 - 0.5) * 20e-9, 0.0)
        sim = Simulation(size=size, resolution=1 / 20e-9, pml_layers=4, courant_factor=0.5)
        src = ElectricDipole(position=(0.3e-6, 0.4e-6, 0.0), polarization="z", frequency=193e12,
                             pulse=True, pulse_width=4e-15)
        mon = FieldMonitor(center=(0.6e-6, 0.4e-6, 0.0), size=(0.0, 0.5e-6, 0.0), components=["Ez"],
                           time_domain=False, frequencies=[193e12])
        sim.add_source(src)
        sim.add_monitor(mon)
        for _ in range(120):
            sim.step()
        g = O.OracleGrid(size, 1 / 20e-9, 4)
        o = O.OracleFDTD(g, g.suggest_dt(0.5), cpml_layers=4)
        b = g.region_bounds((0.3e-6, 0.4e-6, 0.0), (0, 0, 0))
        o.add_source("Ez", g.component_indices("Ez", *b), O.gaussian_pulse(193e12, 4e-15))
        o.run(120)
        got = np.asarray(sim.fields["Ez"])
        assert np.linalg.norm(got - o.F["Ez"]) / np.linalg.norm(o.F["Ez"]) <= 1e-5
        assert np.abs(mon.get_frequency_data("Ez", 193e12)).max() > 0
    finally:
        prismo.set_backend("numpy")


def test_reference_gaussian_beam_is_adapted(prismo):
    """A reference GaussianBeamSource becomes the device source with the same
    region, profile parameters and waveform (no GPU needed)."""
    from prismo.sources.gaussian import GaussianBeamSource as RefBeam

    from prismo_gb300 import plugin
    from prismo_gb300 import sources as S

    ref = RefBeam(center=(0.2e-6, 0.2e-6, 0.2e-6), size=(0.0, 0.2e-6, 0.2e-6), direction="x", polarization="z",
                  frequency=193e12, beam_waist=0.1e-6, pulse=True, pulse_width=4e-15)
    out = plugin._adapt_source(ref)
    assert isinstance(out, S.GaussianBeamSource)
    assert (out.direction, out.polarization, out.beam_waist, out.frequency) == ("x", "z", 0.1e-6, 193e12)
    assert out.waveform is ref.waveform
    assert tuple(out.center) == tuple(ref.center) and tuple(out.size) == tuple(ref.size)
