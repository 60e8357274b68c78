"""GPU TFSF plane source against the oracle (1D auxiliary line, corrections on the
H plane before the E pass and on the E plane after it).

Tolerances: float64 |err| <= 1e-11 x max|field|; float32 relative L2 <= 1e-5."""

import numpy as np
import pytest

from oracle import fdtd64 as O

pytestmark = pytest.mark.gpu

COMPS = O.COMPONENTS


@pytest.fixture(scope="module")
def torch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("fused", [True, False])
@pytest.mark.parametrize("direction,pol", [(-1, "x"), (1, "y")])
def test_tfsf_matches_oracle(torch, direction, pol, fused):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    g = O.OracleGrid.from_total(24, 22, 60, 20e-9, 4)
    dt = g.suggest_dt(0.5)
    eps = np.ones(g.dims)
    eps[:, :, :20] = 4.0  # a half-space below the plane
    wf = O.gaussian_pulse(193e12, 3e-15)
    k0 = 40 if direction < 0 else 25
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=4,
                     tfsf=O.TFSFPlane(k0=k0, direction=direction, polarization=pol, waveform=wf))
    n = 160
    o.run(n)
    for prec in ("fp64", "fp32"):
        eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=False, precision=prec, material_arrays={"eps_rel": eps},
                         pml=PMLParams(thickness=4))
        eng.set_tfsf(k0, direction, pol, wf)
        eng.set_fused_extras(fused)
        t = np.cumsum(np.full(n, dt))
        eng.step(n, np.array([wf(x) for x in t])[:, None])
        assert eng.check_status() == 0
        for c in COMPS:
            got = eng.component(c).double().cpu().numpy()
            ref = o.F[c]
            if prec == "fp64":
                np.testing.assert_allclose(got, ref, rtol=0, atol=1e-11 * max(np.abs(ref).max(), 1e-300),
                                           err_msg=c)
            else:
                assert rel(got, ref) <= 1e-5, (c, rel(got, ref))
        eng.close()
