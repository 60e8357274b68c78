"""Benchmark configurations end to end on the GPU.

* 2D TE drop-in (500 x 250, 20-cell CPML, 3000 steps, slab waveguide, line
  source, 11-frequency DFT line): float64 kernels vs the float64 oracle
  (|err| <= 1e-11 x max), float32 vs the oracle (fields rel L2 <= 1e-5, DFT
  <= 1e-4).
* 3D 256^3 FP32 CPML workload at full size and length (2000 steps): float32
  against the float64 kernels (which match the oracle to 1e-12 on smaller grids):
  rel L2 <= 1e-5 per field component.
"""

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


def test_2d_te_dropin_config_full_size(torch):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams
    from prismo_gb300.workloads import CONFIG_2D, config_2d_layout

    cfg = CONFIG_2D
    g = O.OracleGrid.from_total(*cfg["dims"], cfg["dx"], cfg["cpml"])
    dt = g.suggest_dt(cfg["courant"])
    eps, src, mon, freqs = config_2d_layout()
    wf = O.gaussian_pulse(cfg["pulse_f0"], cfg["pulse_width"])
    n = cfg["steps"]
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=cfg["cpml"])
    o.add_source("Ez", src, wf)
    d = o.add_dft("Ez", mon, freqs)
    o.run(n)
    t = np.cumsum(np.full(n, dt))
    amps = np.array([wf(x) for x in t])[:, None]
    for prec in ("fp64", "fp32"):
        eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=True, precision=prec, material_arrays={"eps_rel": eps},
                         pml=PMLParams(thickness=cfg["cpml"]))
        eng.add_source("Ez", eng.offsets("Ez", src), None, wf)
        m = eng.add_dft("Ez", eng.offsets("Ez", mon), freqs, t0=dt)
        eng.step(n, amps)
        assert eng.check_status() == 0
        got = eng.dft_result(m).cpu().numpy()
        want = o.dfts[d].data.reshape(len(freqs), -1)
        for c in ("Ez", "Hx", "Hy"):
            f = eng.component(c).double().cpu().numpy()
            if prec == "fp64":
                np.testing.assert_allclose(f, o.F[c], rtol=0, atol=1e-11 * np.abs(o.F[c]).max(), err_msg=c)
            else:
                assert rel(f, o.F[c]) <= 1e-5, (c, rel(f, o.F[c]))
        for i in range(len(freqs)):
            assert rel(got[i], want[i]) <= 1e-4, (prec, i, rel(got[i], want[i]))
        eng.close()


def test_3d_fp32_workload_full_size_vs_fp64(torch):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.grid import YeeGrid
    from prismo_gb300.pml import PMLParams
    from prismo_gb300.sources import GaussianPulse
    from prismo_gb300.workloads import CONFIG_3D, boxes_3d

    cfg = CONFIG_3D
    dims = cfg["dims"]
    grid = YeeGrid.from_total(dims, cfg["dx"], cfg["cpml"])
    dt = grid.suggest_time_step(cfg["courant"])
    eps = boxes_3d(dims, seed=cfg["seed"])
    wf = GaussianPulse(cfg["pulse_f0"], cfg["pulse_width"])
    n = cfg["steps"]
    c = tuple(d // 2 for d in dims)
    idx = tuple(np.array([v]).reshape(1, 1, 1) for v in c)
    amps = np.asarray(wf(np.cumsum(np.full(n, dt))), dtype=np.float64).reshape(n, 1)
    out = {}
    for prec in ("fp64", "fp32"):
        eng = FDTDEngine(grid.dimensions, grid.spacing, dt, is_2d=False, precision=prec,
                         material_arrays={"eps_rel": eps}, pml=PMLParams(thickness=cfg["cpml"]))
        eng.add_source("Ez", eng.offsets("Ez", idx), None, wf)
        eng.step(n, amps)
        assert eng.check_status() == 0
        out[prec] = {k: eng.component(k).double() for k in COMPS}
        eng.close()
    errs = {k: float((out["fp32"][k] - out["fp64"][k]).norm() / out["fp64"][k].norm()) for k in COMPS}
    print("fp32 vs fp64 rel L2 after 2000 steps:", errs)
    for k in COMPS:
        assert errs[k] <= 1e-5, (k, errs[k])


def test_2d_config_batched_route_equals_engine_kernels(torch):
    """The 2D TE configuration through FDTDEngine runs on the batched kernel
    (K time steps per launch); the same engine with that route off runs the
    per-step kernels: the two float32 paths round differently (explicit
    roundings against contracted multiply-adds) and agree to 1e-5 in the fields
    and the DFT line, the bar both meet against the float64 oracle."""
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams
    from prismo_gb300.workloads import CONFIG_2D, config_2d_layout

    cfg = CONFIG_2D
    g = O.OracleGrid.from_total(*cfg["dims"], cfg["dx"], cfg["cpml"])
    dt = g.suggest_dt(cfg["courant"])
    eps, src, mon, freqs = config_2d_layout()
    wf = O.gaussian_pulse(cfg["pulse_f0"], cfg["pulse_width"])
    n = cfg["steps"]
    amps = np.array([wf(x) for x in np.cumsum(np.full(n, dt))])[:, None]
    out = []
    for route in (False, True):
        eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=True, precision="fp32", material_arrays={"eps_rel": eps},
                         pml=PMLParams(thickness=cfg["cpml"]), batch_route=route)
        eng.add_source("Ez", eng.offsets("Ez", src), None, wf)
        m = eng.add_dft("Ez", eng.offsets("Ez", mon), freqs, t0=dt)
        eng.step(n // 2, amps[: n // 2])  # two calls: the amplitude rows continue
        eng.step(n - n // 2, amps[n // 2:])
        assert (eng._route is not None) == route
        assert eng.check_status() == 0
        out.append(({c: eng.component(c).double().cpu().numpy() for c in ("Ez", "Hx", "Hy")},
                    eng.dft_result(m).cpu().numpy(), eng.launch_count()))
        eng.close()
    for c in ("Ez", "Hx", "Hy"):
        assert rel(out[1][0][c], out[0][0][c]) <= 1e-5, (c, rel(out[1][0][c], out[0][0][c]))
    assert rel(out[1][1], out[0][1]) <= 1e-5
    print("launches: per-step kernels", out[0][2], "batched route", out[1][2])
