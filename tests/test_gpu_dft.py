"""GPU DFT monitors (batched samples, float64 phase recurrence, Kahan float32
sums) against the oracle's FieldMonitor DFT (monitors/field.py:138-143).

Tolerance: relative L2 of the complex spectrum <= 1e-4 per (component, frequency)
set, for float32 fields."""

import numpy as np
import pytest

from oracle import fdtd64 as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("nsteps", [150, 160])
def test_dft_3d_plane_matches_oracle(torch, nsteps):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    g = O.OracleGrid.from_total(40, 36, 44, 20e-9, 4)
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(4)
    eps = rng.uniform(1.0, 4.0, size=g.dims)
    wf = O.gaussian_pulse(193e12, 2e-15)
    freqs = [150e12, 193e12, 230e12, 300e12]
    src = g.component_indices("Ez", 12, 13, 17, 18, 21, 22)
    plane_ez = g.component_indices("Ez", 28, 29, 0, 36, 0, 44)
    plane_hy = g.component_indices("Hy", 28, 29, 0, 36, 0, 44)
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=4)
    o.add_source("Ez", src, wf)
    d_ez = o.add_dft("Ez", plane_ez, freqs)
    d_hy = o.add_dft("Hy", plane_hy, freqs)
    o.run(nsteps)
    eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=False, precision="fp32", material_arrays={"eps_rel": eps},
                     pml=PMLParams(thickness=4))
    eng.add_source("Ez", eng.offsets("Ez", src), None, wf)
    m_ez = eng.add_dft("Ez", eng.offsets("Ez", plane_ez), freqs, t0=dt)
    m_hy = eng.add_dft("Hy", eng.offsets("Hy", plane_hy), freqs, t0=dt)
    t = np.cumsum(np.full(nsteps, dt))
    eng.step(nsteps, np.array([wf(x) for x in t])[:, None])
    got_ez = eng.dft_result(m_ez).cpu().numpy()
    got_hy = eng.dft_result(m_hy).cpu().numpy()
    assert eng.check_status() == 0
    want_ez = o.dfts[d_ez].data.reshape(len(freqs), -1)
    want_hy = o.dfts[d_hy].data.reshape(len(freqs), -1)
    for f in range(len(freqs)):
        assert rel(got_ez[f], want_ez[f]) <= 1e-4, (f, rel(got_ez[f], want_ez[f]))
        assert rel(got_hy[f], want_hy[f]) <= 1e-4, (f, rel(got_hy[f], want_hy[f]))
    eng.close()


def test_dft_2d_line_matches_oracle(torch):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    g = O.OracleGrid.from_total(90, 60, 1, 20e-9, 8)
    dt = g.suggest_dt(0.5)
    eps = np.full(g.dims, 2.085)
    eps[:, 25:35, :] = 12.11
    wf = O.gaussian_pulse(193e12, 5e-15)
    freqs = list(299792458.0 / np.linspace(1.5e-6, 1.6e-6, 11))
    src = g.component_indices("Ez", 10, 11, 24, 36, 0, 1)
    line = g.component_indices("Ez", 70, 71, 0, 60, 0, 1)
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=8)
    o.add_source("Ez", src, wf)
    d = o.add_dft("Ez", line, freqs)
    n = 700
    o.run(n)
    eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=True, precision="fp32", material_arrays={"eps_rel": eps},
                     pml=PMLParams(thickness=8))
    eng.add_source("Ez", eng.offsets("Ez", src), None, wf)
    m = eng.add_dft("Ez", eng.offsets("Ez", line), freqs, t0=dt)
    t = np.cumsum(np.full(n, dt))
    eng.step(n, np.array([wf(x) for x in t])[:, None])
    got = eng.dft_result(m).cpu().numpy()
    want = o.dfts[d].data.reshape(len(freqs), -1)
    for f in range(len(freqs)):
        assert rel(got[f], want[f]) <= 1e-4, (f, rel(got[f], want[f]))
    eng.close()
