"""GPU dispersive (ADE) updates against the oracle: Lorentz, Drude and Debye poles
coupled to E (the reference updates P/J in isolation, materials/ade.py:100-160;
the coupling is defined in the oracle's ade_e_coefficients).

Tolerances as for the stepper: float64 |err| <= 1e-11 x max|field|, float32
relative L2 <= 1e-5."""

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


def poles(dt):
    return [O.drude_coeffs(1.37e16, 1.0e14, dt), O.lorentz_coeffs(1.2, 4.0e15, 2.0e14, dt),
            O.lorentz_coeffs(0.7, 5.5e15, 4.0e14, dt)]


@pytest.mark.parametrize("is2d,fused", [(False, True), (False, False), (True, False)])
def test_ade_matches_oracle(torch, is2d, fused):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    if is2d:
        g = O.OracleGrid.from_total(60, 50, 1, 20e-9, 5)
        box = (0, 60, 0, 20, 0, 1)
        src = g.component_indices("Ez", 30, 31, 35, 36, 0, 1)
        comp = "Ez"
    else:
        g = O.OracleGrid.from_total(30, 28, 34, 20e-9, 4)
        box = (0, 30, 0, 28, 0, 14)
        src = g.component_indices("Ex", 15, 16, 14, 15, 24, 25)
        comp = "Ex"
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(8)
    eps = rng.uniform(1.0, 4.0, size=g.dims)
    pl = poles(dt)
    pl.append(O.debye_coeffs(5.0, 2.0, 3e-15, dt))
    wf = O.gaussian_pulse(193e12, 2e-15)
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=4,
                     ade=[O.ADERegion(box=box, eps_inf=1.0, poles=pl)])
    o.add_source(comp, src, wf)
    n = 80
    o.run(n)
    for prec in ("fp64", "fp32"):
        eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=is2d, precision=prec, material_arrays={"eps_rel": eps},
                         pml=PMLParams(thickness=4))
        eng.set_dispersive([(box, 1.0, pl)])
        eng.set_fused_extras(fused)
        eng.add_source(comp, eng.offsets(comp, src), None, wf)
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
