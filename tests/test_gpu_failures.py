"""Failure detection without a GPU fault: a NaN written into one field buffer
from the host before stepping must come back as PC_STATUS_NONFINITE and a
``FloatingPointError`` on every stepping path (fused 3D, split 3D, 2D, the
dispersive E update), and in the batched sweep it must mark only the instance
it was written into, whose design is then re-run on the per-simulation path."""

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


def _engine(dims, sched, cpml=4, is_2d=False, precision="fp32"):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    g = O.OracleGrid.from_total(*dims, 20e-9, cpml)
    dt = g.suggest_dt(0.5)
    eps = np.random.default_rng(1).uniform(1.0, 4.0, size=g.dims)
    return FDTDEngine(g.dims, g.spacing, dt, is_2d=is_2d, precision=precision, sched=sched,
                      material_arrays={"eps_rel": eps}, pml=PMLParams(thickness=cpml))


@pytest.mark.parametrize("case", ["fused3d", "split3d", "split2d", "fused3d_fp64"])
def test_nan_in_fields_raises(torch, case):
    from prismo_gb300 import _lib

    if case == "split2d":
        eng = _engine((40, 36, 1), "split", is_2d=True)
        eng.component("Hx")[20, 17] = float("nan")
    else:
        eng = _engine((40, 36, 44), "split" if case == "split3d" else "fused",
                      precision="fp64" if case.endswith("fp64") else "fp32")
        eng.component("Hy")[20, 17, 21] = float("nan")
    eng.step(3)
    st = eng.status()  # reads and clears the word
    assert st & _lib.PC_STATUS_NONFINITE, st
    assert not st & (_lib.PC_STATUS_BOUNDS | _lib.PC_STATUS_TIMEOUT), st
    eng.step(1)  # the NaN is still in the fields: the next step flags it again
    with pytest.raises(FloatingPointError):
        eng.check_status()
    eng.close()


def test_clean_run_reports_no_failure(torch):
    eng = _engine((40, 36, 44), "fused")
    eng.component("Ez")[20, 17, 21] = 1.0
    eng.step(5)
    assert eng.check_status() == 0
    eng.close()


def test_nan_in_dispersive_region_raises(torch):
    from prismo_gb300.workloads import build_dispersive_engine

    eng, info = build_dispersive_engine((40, 36, 64), precision="fp32", cpml=6, z_metal=24, ridge_width=0.3e-6)
    eng.component("Hx")[20, 17, 10] = float("nan")  # inside the metal (z < 24)
    wf, dt = info["waveform"], info["dt"]
    eng.step(2, wf((np.arange(2) + 1) * dt)[:, None])
    with pytest.raises(FloatingPointError):
        eng.check_status()
    eng.close()


def test_batched_sweep_marks_only_the_poisoned_instance_and_reruns_it(torch):
    from prismo_gb300 import sweep as S

    designs = [S.design_from_params([0.3, 0.2, 0.1], nx=400, ny=200, seed=-1),
               S.design_from_params([0.8, 0.7, 0.6], nx=400, ny=220, seed=-2),
               S.design_from_params([0.5, 0.4, 0.3], nx=420, ny=210, seed=-3)]
    nsteps, nf = 480, 8

    def poison(B):  # design 1's coupler instance (instances: coupler, normalisation per design)
        ez, _, _ = B.fields(2)
        ez[150, 100] = float("nan")

    clean = S.batched_sweep(designs, nsteps=nsteps, nfreq=nf, autotune=False)
    assert clean.rerun == [] and clean.failed == []
    r = S.batched_sweep(designs, nsteps=nsteps, nfreq=nf, autotune=False, prepare=poison)
    assert r.rerun == [1] and r.failed == []
    assert np.isfinite(r.S).all()
    scale = max(1.0, np.abs(clean.S).max())
    for q in range(len(designs)):  # the re-run design matches the clean batched result
        assert np.abs(r.S[q] - clean.S[q]).max() <= 1e-6 * scale, q
