"""GPU parity of the stepping kernels against the reference fixtures and the oracle.

Tolerances: float64 kernels of the reference stepper must equal the reference
bit for bit; float64 corrected kernels must match the FP64 oracle to 1e-12
(relative to the field maximum); float32 kernels must match to relative L2
<= 1e-5 per component.
"""

import json
import os

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


def make_engine(dims, spacing, dt, is_2d, **kw):
    from prismo_gb300.engine import FDTDEngine

    return FDTDEngine(dims, spacing, dt, is_2d=is_2d, **kw)


def load_fields(eng, init, torch):
    for c in COMPS:
        eng.component(c).copy_(torch.from_numpy(np.asarray(init[c])).to(eng.device, eng.dtype))


def read_fields(eng):
    return {c: eng.component(c).double().cpu().numpy() for c in COMPS}


def rel_l2(a, b):
    n = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (n if n > 0 else 1.0)


@pytest.mark.parametrize("name", ["ref_l0_3d.npz", "ref_l0_2d.npz"])
def test_reference_stepper_fp64_is_bit_exact(torch, golden_dir, name):
    z = np.load(os.path.join(golden_dir, name))
    meta = json.loads(str(z["meta"]))
    g = O.OracleGrid(tuple(meta["size"]), meta["resolution"], meta["layers"])
    mats = {k: z[k] for k in ("eps_rel", "mu_rel", "sigma_e", "sigma_m")}
    eng = make_engine(g.dims, g.spacing, meta["dt"], g.is_2d, precision="fp64", mode="legacy",
                      material_arrays=mats)
    load_fields(eng, {c: z[f"init_{c}"] for c in COMPS}, torch)
    eng.step(meta["nsteps"])
    out = read_fields(eng)
    for c in COMPS:
        np.testing.assert_array_equal(out[c], z[f"out_{c}"], err_msg=c)
    eng.close()


def _random_case(dims, is_2d, seed, lossy):
    rng = np.random.default_rng(seed)
    nx, ny, nz = dims
    d = 20e-9
    if is_2d:
        g = O.OracleGrid.from_total(nx, ny, 1, d, 3)
    else:
        g = O.OracleGrid.from_total(nx, ny, nz, d, 3)
    mats = {"eps_rel": rng.uniform(1.0, 12.0, size=g.dims)}
    if lossy:
        mats["sigma_e"] = rng.uniform(0.0, 3e4, size=g.dims)
        mats["mu_rel"] = rng.uniform(1.0, 1.5, size=g.dims)
        mats["sigma_m"] = rng.uniform(0.0, 3e3, size=g.dims)
    init = {}
    for c in COMPS:
        init[c] = rng.standard_normal(g.shape(c)) * (1.0 if c[0] == "E" else 1 / 377.0)
    # respect the stepper invariants: boundary H entries that are never updated
    return g, mats, init


@pytest.mark.parametrize("sched", ["split", "fused"])
@pytest.mark.parametrize("lossy", [False, True])
@pytest.mark.parametrize("cpml", [0, 4])
def test_corrected_3d_matches_oracle(torch, sched, lossy, cpml):
    g, mats, init = _random_case((37, 29, 45), False, seed=11 + cpml + lossy, lossy=lossy)
    dt = g.suggest_dt(0.5)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=cpml)
    for c in COMPS:
        o.F[c][...] = init[c]
    nsteps = 20
    o.run(nsteps)
    from prismo_gb300.pml import PMLParams

    pml = PMLParams(thickness=cpml) if cpml else None
    for prec in ("fp64", "fp32"):
        eng = make_engine(g.dims, g.spacing, dt, False, precision=prec, sched=sched, material_arrays=mats, pml=pml)
        load_fields(eng, init, torch)
        eng.step(nsteps)
        out = read_fields(eng)
        assert eng.check_status() == 0
        for c in COMPS:
            ref = o.F[c]
            if prec == "fp64":
                np.testing.assert_allclose(out[c], ref, rtol=0, atol=1e-12 * np.abs(ref).max(), err_msg=c)
            else:
                assert rel_l2(out[c], ref) <= 1e-5, (c, rel_l2(out[c], ref))
        eng.close()


@pytest.mark.parametrize("lossy", [False, True])
@pytest.mark.parametrize("cpml", [0, 5])
def test_corrected_2d_matches_oracle(torch, lossy, cpml):
    g, mats, init = _random_case((53, 41, 1), True, seed=21 + cpml + lossy, lossy=lossy)
    dt = g.suggest_dt(0.5)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=cpml)
    for c in COMPS:
        o.F[c][...] = init[c]
    nsteps = 30
    o.run(nsteps)
    from prismo_gb300.pml import PMLParams

    pml = PMLParams(thickness=cpml) if cpml else None
    for prec in ("fp64", "fp32"):
        eng = make_engine(g.dims, g.spacing, dt, True, precision=prec, material_arrays=mats, pml=pml)
        load_fields(eng, init, torch)
        eng.step(nsteps)
        out = read_fields(eng)
        assert eng.check_status() == 0
        for c in COMPS:
            ref = o.F[c]
            if prec == "fp64":
                np.testing.assert_allclose(out[c], ref, rtol=0, atol=1e-12 * np.abs(ref).max(), err_msg=c)
            else:
                assert rel_l2(out[c], ref) <= 1e-5, (c, rel_l2(out[c], ref))
        eng.close()


def test_fused_equals_split_fp32_long_run(torch):
    """The fused and split schedules implement the same arithmetic."""
    g, mats, init = _random_case((70, 66, 100), False, seed=5, lossy=False)
    dt = g.suggest_dt(0.5)
    from prismo_gb300.pml import PMLParams

    outs = []
    for sched in ("split", "fused"):
        eng = make_engine(g.dims, g.spacing, dt, False, precision="fp32", sched=sched, material_arrays=mats,
                          pml=PMLParams(thickness=6))
        load_fields(eng, init, torch)
        eng.step(101)
        outs.append(read_fields(eng))
        assert eng.check_status() == 0
        eng.close()
    for c in COMPS:
        assert rel_l2(outs[1][c], outs[0][c]) <= 1e-6, c


def test_point_source_matches_oracle(torch):
    g = O.OracleGrid.from_total(31, 27, 25, 20e-9, 4)
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(3)
    mats = {"eps_rel": rng.uniform(1.0, 4.0, size=g.dims)}
    wf = O.gaussian_pulse(193e12, 2e-15)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=4)
    idx = g.component_indices("Ez", 15, 16, 13, 14, 12, 13)
    o.add_source("Ez", idx, wf)
    n = 40
    o.run(n)
    from prismo_gb300.pml import PMLParams

    for prec in ("fp64", "fp32"):
        eng = make_engine(g.dims, g.spacing, dt, False, precision=prec, material_arrays=mats,
                          pml=PMLParams(thickness=4))
        eng.add_source("Ez", eng.offsets("Ez", idx), None, wf)
        t = np.cumsum(np.full(n, dt))
        eng.step(n, np.array([wf(x) for x in t])[:, None])
        out = read_fields(eng)
        assert eng.check_status() == 0
        for c in COMPS:
            tol = 1e-12 if prec == "fp64" else 1e-5
            assert rel_l2(out[c], o.F[c]) <= tol, (prec, c, rel_l2(out[c], o.F[c]))
        eng.close()


@pytest.mark.parametrize("chunk", [0, 5, 7])
def test_fused_chunking_with_cpml_slabs(torch, chunk):
    """x-chunks of every length end on the last plane with y/z CPML slabs active."""
    from prismo_gb300 import _lib
    from prismo_gb300.pml import PMLParams

    g, mats, init = _random_case((29, 35, 41), False, seed=9, lossy=False)
    dt = g.suggest_dt(0.5)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=5)
    for c in COMPS:
        o.F[c][...] = init[c]
    o.run(12)
    eng = make_engine(g.dims, g.spacing, dt, False, precision="fp32", sched="fused", material_arrays=mats,
                      pml=PMLParams(thickness=5))
    eng.set_time_blocking(0)  # the fused schedule's own chunking
    if chunk:
        _lib.check(eng.lib.pc_set_tuning(eng.ctx, _lib.PC_TUNE_FUSED_CHUNK, chunk))
    load_fields(eng, init, torch)
    eng.step(12)
    out = read_fields(eng)
    assert eng.check_status() == 0
    for c in COMPS:
        assert rel_l2(out[c], o.F[c]) <= 1e-5, c
    eng.close()


@pytest.mark.parametrize("chunk,edge,split,unified", [(0, 0, 1, 0), (9, 0, 1, 0), (16, 5, 1, 0), (9, 0, 2, 0),
                                                     (9, 0, 2, 1), (16, 5, 1, 1), (0, 0, 0, 0)])
def test_fused_plain_and_cpml_item_classes(torch, chunk, edge, split, unified):
    """Every item class in one step: tiles clear of every slab (variant without
    CPML code), in float32 tiles that touch only the x slabs (inner tiles of the
    end chunks), only a y slab (j0 = 0, 48, 64 at k0 = 32), only a z slab (j0 = 16,
    32 at k0 = 0, 64, 96) with their single-axis variants, the rest (and every
    CPML item in float64) with the general one, concurrently; split 2 adds the
    two-axis variants, split 0 leaves only the general one; `unified` runs every
    class from one launch; tiles whose +1 H
    halo row/column lands exactly on the first slab row/column (ny - t = 48 + 16,
    nz - t = 64 + 32)."""
    from prismo_gb300 import _lib
    from prismo_gb300.pml import PMLParams

    g, mats, init = _random_case((80, 72, 104), False, seed=11, lossy=False)
    dt = g.suggest_dt(0.5)
    o = O.OracleFDTD(g, dt, mats, cpml_layers=8)
    for c in COMPS:
        o.F[c][...] = init[c]
    o.run(30)
    for prec in ("fp64", "fp32"):
        eng = make_engine(g.dims, g.spacing, dt, False, precision=prec, sched="fused", material_arrays=mats,
                          pml=PMLParams(thickness=8))
        eng.set_time_blocking(0)  # the fused schedule's item classes
        if chunk:
            eng.set_chunk(chunk, edge)  # edge: chunk length of the tiles on a y/z slab
        eng.set_split(split, bool(unified))
        load_fields(eng, init, torch)
        eng.step(30)
        out = read_fields(eng)
        assert eng.check_status() == 0
        for c in COMPS:
            tol = 1e-12 if prec == "fp64" else 1e-5
            assert rel_l2(out[c], o.F[c]) <= tol, (prec, c, rel_l2(out[c], o.F[c]))
        eng.close()


@pytest.mark.parametrize("is2d", [True, False])
def test_captured_time_loop_matches_eager_steps(torch, is2d):
    """pc_step replays graphs of 64 steps (sources read their rows from a refilled
    table; DFT rings flush inside the graph): bit-identical to per-step launches,
    also across a change of configuration between calls (a source added later)."""
    from prismo_gb300.pml import PMLParams

    if is2d:
        g = O.OracleGrid.from_total(96, 70, 1, 20e-9, 8)
        idx = g.component_indices("Ez", 30, 31, 20, 50, 0, 1)
        idx2 = g.component_indices("Ez", 60, 61, 30, 31, 0, 1)
        comp = "Ez"
    else:
        g = O.OracleGrid.from_total(40, 36, 48, 20e-9, 6)
        idx = g.component_indices("Ez", 20, 21, 18, 19, 24, 25)
        idx2 = g.component_indices("Ex", 12, 13, 10, 11, 30, 31)
        comp = "Ez"
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(4)
    mats = {"eps_rel": rng.uniform(1.0, 4.0, size=g.dims)}
    wf = O.gaussian_pulse(193e12, 2e-15)
    mon = g.component_indices(comp, 10, 30, 10, 30, 0, 1) if is2d else g.component_indices(comp, 10, 30, 10, 20, 20, 21)
    freqs = np.linspace(180e12, 200e12, 5)
    outs = []
    for graph_steps in (0, 64):
        eng = make_engine(g.dims, g.spacing, dt, is2d, precision="fp32", material_arrays=mats,
                          pml=PMLParams(thickness=6 if not is2d else 8), batch_route=False)
        eng.set_graph_steps(graph_steps)
        eng.add_source(comp, eng.offsets(comp, idx), None, wf)
        m = eng.add_dft(comp, eng.offsets(comp, mon), freqs, t0=dt)
        t = (np.arange(300) + 1) * dt
        eng.step(150, np.array([wf(x) for x in t[:150]])[:, None])
        # a second source from step 150 on: the captured graph must be re-captured
        eng.add_source("Ex" if not is2d else "Ez", eng.offsets("Ex" if not is2d else "Ez", idx2), None, wf)
        a2 = np.stack([np.array([wf(x) for x in t[150:]]), 0.5 * np.array([wf(x) for x in t[150:]])], axis=1)
        eng.step(150, a2)
        assert eng.check_status() == 0
        outs.append((read_fields(eng), eng.dft_result(m).cpu().numpy(), eng.launch_count()))
        eng.close()
    for c in (("Ez", "Hx", "Hy") if is2d else COMPS):
        assert np.array_equal(outs[0][0][c], outs[1][0][c]), c
    assert np.array_equal(outs[0][1], outs[1][1])
