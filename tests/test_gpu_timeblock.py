"""The temporally blocked 3D stepper (two or one time steps per launch, float32)
against the float64 oracle: every item class (interior tiles, tiles at the
domain boundary without CPML, tiles on the x, y or z slabs and on several),
every x-chunk length, odd step counts (a one-step launch finishes them), soft
sources on tile and chunk borders (fused into the kernel), captured time loops,
and agreement with the one-step fused schedule.  Tolerance: relative L2 <= 1e-5
per component against the oracle."""

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


def rel_l2(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


def _case(dims, seed, cpml):
    rng = np.random.default_rng(seed)
    g = O.OracleGrid.from_total(*dims, 20e-9, max(cpml, 1))
    mats = {"eps_rel": rng.uniform(1.0, 12.0, size=g.dims)}
    init = {c: rng.standard_normal(g.shape(c)) * (1.0 if c[0] == "E" else 1 / 377.0) for c in COMPS}
    return g, mats, init


def _engine(torch, g, dt, mats, init, cpml, steps, chunk=0):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=False, precision="fp32", sched="fused", material_arrays=mats,
                     pml=PMLParams(thickness=cpml) if cpml else None)
    eng.set_time_blocking(steps, chunk)
    if init is not None:
        for c in COMPS:
            eng.component(c).copy_(torch.from_numpy(np.asarray(init[c])).to(eng.device, eng.dtype))
    return eng


def _read(eng):
    return {c: eng.component(c).double().cpu().numpy() for c in COMPS}


@pytest.mark.parametrize("steps", [2, 1])
@pytest.mark.parametrize("cpml", [0, 4])
@pytest.mark.parametrize("chunk", [0, 5, 16])
def test_blocked_stepper_matches_oracle(torch, steps, cpml, chunk):
    g, mats, init = _case((37, 29, 45), 31 + cpml + chunk, cpml)
    dt = g.suggest_dt(0.5)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=cpml)
    for c in COMPS:
        o.F[c][...] = init[c]
    n = 21  # odd: the last step runs as a one-step launch
    o.run(n)
    eng = _engine(torch, g, dt, mats, init, cpml, steps, chunk)
    eng.step(n)
    out = _read(eng)
    assert eng.check_status() == 0
    for c in COMPS:
        assert rel_l2(out[c], o.F[c]) <= 1e-5, (c, rel_l2(out[c], o.F[c]))
    eng.close()


def test_blocked_stepper_every_item_class(torch):
    """80 x 72 x 104 with an 8-cell CPML and 16 x 32 tiles: interior tiles clear of
    every slab, tiles on one, two and three axes' slabs, in one launch."""
    g, mats, init = _case((80, 72, 104), 11, 8)
    dt = g.suggest_dt(0.5)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=8)
    for c in COMPS:
        o.F[c][...] = init[c]
    o.run(30)
    for chunk in (0, 9):
        eng = _engine(torch, g, dt, mats, init, 8, 2, chunk)
        eng.step(30)
        out = _read(eng)
        assert eng.check_status() == 0
        for c in COMPS:
            assert rel_l2(out[c], o.F[c]) <= 1e-5, (chunk, c, rel_l2(out[c], o.F[c]))
        eng.close()


def test_fused_sources_on_tile_and_chunk_borders(torch):
    """Soft E sources at points that lie in the halo of neighbouring tiles and
    chunks (j = 16, k = 32, i = chunk border), several components and weights."""
    g = O.OracleGrid.from_total(70, 50, 72, 20e-9, 6)
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(8)
    mats = {"eps_rel": rng.uniform(1.0, 4.0, size=g.dims)}
    wf = O.gaussian_pulse(193e12, 2e-15)
    wf2 = O.gaussian_pulse(180e12, 3e-15, amplitude=0.7)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=6)
    srcs = [("Ez", g.component_indices("Ez", 32, 33, 16, 17, 32, 33), wf, 1.0),
            ("Ex", g.component_indices("Ex", 31, 32, 15, 17, 31, 33), wf2, 0.5),
            ("Ey", g.component_indices("Ey", 20, 21, 30, 31, 40, 41), wf, -1.3)]
    for comp, idx, w, a in srcs:
        o.add_source(comp, idx, w, weight=a)
    n = 41
    o.run(n)
    t = (np.arange(n) + 1) * dt
    amps = np.stack([np.array([w(x) for x in t]) for _, _, w, _ in srcs], axis=1)
    for steps, chunk in ((2, 0), (2, 32), (1, 0)):
        eng = _engine(torch, g, dt, mats, None, 6, steps, chunk)
        for comp, idx, w, a in srcs:
            off = eng.offsets(comp, idx)
            eng.add_source(comp, off, np.full(off.size, a), w)
        eng.step(n, amps)
        out = _read(eng)
        assert eng.check_status() == 0
        for c in COMPS:
            assert rel_l2(out[c], o.F[c]) <= 1e-5, (steps, chunk, c, rel_l2(out[c], o.F[c]))
        eng.close()


def test_blocked_equals_one_step_schedule(torch):
    """Two steps per launch against the one-step fused schedule over 101 steps."""
    g, mats, init = _case((70, 66, 100), 5, 6)
    dt = g.suggest_dt(0.5)
    outs = []
    for steps in (0, 2):
        eng = _engine(torch, g, dt, mats, init, 6, steps)
        eng.step(101)
        outs.append(_read(eng))
        assert eng.check_status() == 0
        eng.close()
    for c in COMPS:
        assert rel_l2(outs[1][c], outs[0][c]) <= 1e-6, (c, rel_l2(outs[1][c], outs[0][c]))


def test_blocked_captured_loop_equals_eager(torch):
    """Graph replay of two-step launches (amplitude rows refilled per replay) is
    bit-identical to eager launches, and the profiler counts two steps per launch."""
    g = O.OracleGrid.from_total(40, 36, 48, 20e-9, 6)
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(4)
    mats = {"eps_rel": rng.uniform(1.0, 4.0, size=g.dims)}
    wf = O.gaussian_pulse(193e12, 2e-15)
    idx = g.component_indices("Ez", 20, 21, 18, 19, 24, 25)
    t = (np.arange(200) + 1) * dt
    amps = np.array([wf(x) for x in t])[:, None]
    outs = []
    for graph_steps in (0, 64):
        eng = _engine(torch, g, dt, mats, None, 6, 2)
        eng.set_graph_steps(graph_steps)
        eng.add_source("Ez", eng.offsets("Ez", idx), None, wf)
        if graph_steps == 0:
            eng.profile(True)
        eng.step(200, amps)
        if graph_steps == 0:
            ms, launches, steps = eng.profile_read()
            assert launches == 100 and steps == 200, (launches, steps)
        assert eng.check_status() == 0
        outs.append(_read(eng))
        eng.close()
    for c in COMPS:
        assert np.array_equal(outs[0][c], outs[1][c]), c
