"""Batched 2D sweep (pc_batch_* through prismo_gb300.sweep) on the GPU.

* every instance of a batch equals the same simulation run alone through the
  single-simulation 2D engine (fields rel L2 <= 1e-6, port DFT <= 1e-6);
* all kernel variants (tile shape, steps per pass) and graph replay vs eager
  passes give bit-identical fields and spectra;
* S-parameters of full-length (4000-step) couplers against the float64 oracle:
  max |S_gpu - S_oracle| <= 1e-3 (the sweep's bar), reported per design;
* batched S-parameters equal the serial per-design engine path (<= 1e-6).
"""

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


def small_instances(cpml=10):
    """Three uneven small guides with a mode-profile source and two ports each."""
    from prismo_gb300 import sweep as S

    out = []
    for q, (nx, ny) in enumerate(((150, 90), (203, 131), (97, 77))):
        eps = S.fill_eps(nx, ny, [(0, nx * S.DX, (ny / 2 - 8 - q) * S.DX, (ny / 2 + 5) * S.DX)], S.DX)
        y0, n = ny // 2 - 14, 26
        prof = np.hanning(n + 2)[1:-1]
        src = S.Port(cpml + 5, y0, n, prof)
        ports = [S.Port(cpml + 12, y0, n, prof), S.Port(nx - cpml - 8, y0 - 2, n + 3, np.ones(n + 3))]
        out.append(S.Instance(eps, src, ports))
    return out


def single_engine_run(inst, nsteps, freqs, dt, cpml):
    from prismo_gb300 import sweep as S
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.pml import PMLParams

    nx, ny = inst.eps.shape
    eng = FDTDEngine((nx, ny, 1), (S.DX, S.DX, S.DX), dt, is_2d=True, precision="fp32",
                     material_arrays={"eps_rel": inst.eps[:, :, None]}, pml=PMLParams(cpml))
    idx = (np.array([[inst.src.x]]), np.arange(inst.src.y0, inst.src.y0 + inst.src.n)[None, :])
    eng.add_source("Ez", eng.offsets("Ez", idx), inst.src.profile, None)
    ids = []
    for p in inst.ports:
        pidx = (np.array([[p.x]]), np.arange(p.y0, p.y0 + p.n)[None, :])
        ids.append(eng.add_dft("Ez", eng.offsets("Ez", pidx), freqs, dt))
    eng.step(nsteps, S.amplitudes(nsteps, dt)[:, None])
    fields = [eng.component(c).double().cpu().numpy() for c in ("Ez", "Hx", "Hy")]
    spec = [eng.dft_result(m).cpu().numpy() for m in ids]
    eng.close()
    return fields, spec


def batch_run(insts, nsteps, freqs, cpml, variant=None, graph_steps=80, chunks=None):
    from prismo_gb300 import sweep as S

    B = S.BatchedFDTD2D(insts, freqs, cpml=cpml, autotune=False, variant=variant if variant is not None else 1,
                        graph_steps=graph_steps)
    B.set_amplitudes(S.amplitudes(nsteps, B.dt))
    for c in chunks or [nsteps]:
        B.step(c)
    assert B.steps_done == nsteps
    fields = [[f.double().cpu().numpy() for f in B.fields(q)] for q in range(len(insts))]
    spec = B.spectra()
    B.close()
    return fields, spec


def test_batch_matches_single_engine(torch):
    from prismo_gb300 import sweep as S

    cpml, n = 10, 240
    insts = small_instances(cpml)
    freqs = S.sweep_freqs(8)
    fields, spec = batch_run(insts, n, freqs, cpml, variant=2, graph_steps=32)
    for q, inst in enumerate(insts):
        f1, s1 = single_engine_run(inst, n, freqs, S.sweep_dt(), cpml)
        for c, a, b in zip(("Ez", "Hx", "Hy"), fields[q], f1):
            assert np.abs(b).max() > 0, (q, c)
            assert rel(a, b) <= 1e-6, (q, c, rel(a, b))
        for k in range(len(inst.ports)):
            assert rel(spec[q][k], s1[k]) <= 1e-6, (q, k, rel(spec[q][k], s1[k]))


def test_variants_and_graph_bit_identical(torch):
    from prismo_gb300 import sweep as S

    cpml, n = 10, 100
    insts = small_instances(cpml)
    freqs = S.sweep_freqs(4)
    ref_f, ref_s = batch_run(insts, n, freqs, cpml, variant=0, graph_steps=0)
    runs = [dict(variant=v, graph_steps=g) for v, (_, _, k) in enumerate(S.BatchedFDTD2D.variants())
            for g in (0, int(np.lcm(16, 2 * k)))]
    runs.append(dict(variant=2, graph_steps=32, chunks=[7, 33, 60]))  # eager / graph / remainder mix
    for r in runs:
        f, s = batch_run(insts, n, freqs, cpml, **r)
        for q in range(len(insts)):
            for a, b in zip(f[q], ref_f[q]):
                assert np.array_equal(a, b), r
            for a, b in zip(s[q], ref_s[q]):
                assert np.array_equal(a, b), r


def oracle_s(layout, nsteps, freqs, dt):
    from prismo_gb300 import sweep as S

    spec = []
    for eps, ports in ((layout.eps, layout.ports), (layout.norm_eps, layout.ports[:1])):
        nx, ny = eps.shape
        g = O.OracleGrid.from_total(nx, ny, 1, S.DX, S.CPML)
        o = O.OracleFDTD(g, dt, {"eps_rel": eps[:, :, None]}, cpml_layers=S.CPML)
        src = layout.src
        wf = O.gaussian_pulse(S.F0, S.PULSE_WIDTH)
        o.add_source("Ez", (np.array([[src.x]]), np.arange(src.y0, src.y0 + src.n)[None, :]), wf,
                     weight=src.profile[None, :])
        ids = [o.add_dft("Ez", (np.array([[p.x]]), np.arange(p.y0, p.y0 + p.n)[None, :]), freqs) for p in ports]
        o.run(nsteps)
        spec.append([o.dfts[m].data.reshape(len(freqs), -1) for m in ids])
    return S.s_parameters(spec[0], spec[1][0], layout)


def test_sparams_vs_oracle_full_length(torch):
    """Two small-footprint couplers (short and long coupling section), 4000 steps.

    4000 steps at Courant 0.5 are 94 fs: the pulse crosses the short coupler
    within the record but only starts to reach the output ports of the long one,
    whose spectra are those of the truncated record (the same for both sides)."""
    from prismo_gb300 import sweep as S

    designs = [S.design_from_params([0.3, 0.2, 0.1], nx=400, ny=200, seed=-1),
               S.design_from_params([0.8, 0.7, 0.6], nx=400, ny=220, seed=-2)]
    layouts = [S.coupler_layout(d) for d in designs]
    freqs = S.sweep_freqs(16)
    res = S.batched_sweep(designs, nsteps=S.STEPS, nfreq=16, autotune=True, layouts=layouts)
    for q, L in enumerate(layouts):
        want = oracle_s(L, S.STEPS, freqs, S.sweep_dt())
        err = np.abs(res.S[q] - want).max()
        print(f"design {q}: max|S| {np.abs(want).max():.3f}  max|dS| {err:.2e}")
        if q == 0:
            assert np.abs(want[1:3]).max() > 0.5  # the pulse reaches the output ports
        assert err <= 1e-3, err


def test_batched_equals_serial_sweep(torch):
    from prismo_gb300 import sweep as S

    designs = [S.coupler_design(s) for s in (3, 11)]
    nsteps = 800
    a = S.batched_sweep(designs, nsteps=nsteps, nfreq=8)
    b = S.serial_sweep(designs, nsteps=nsteps, nfreq=8)
    assert np.abs(a.S - b.S).max() <= 1e-6 * max(1.0, np.abs(b.S).max()), np.abs(a.S - b.S).max()
