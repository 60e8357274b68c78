"""The benchmark configurations at their real sizes against the float64 oracle.

The oracle ran once on the CPU (``tests/golden/make_config_fixtures.py``) and
left compact fixtures: for the 3D grids the full-field L2 norms and sums of the
six components and every 4th cell of nine planes, for the dispersive grid also
the 64-frequency DFT planes (every 8th point of every 8th frequency, and the
per-frequency plane norms and sums), for the seeded couplers their complex
S-parameters.  Each test runs the same configuration on the GPU in float32 and
states the error against float64:

* 256^3 CPML grid, 2000 steps: E and H, each taken as one vector, sampled
  fields rel L2 <= 1e-5 and full-field norms within 1e-5, the Ez probe traces
  within 1e-5 of their peak (Hz of this z-dipole is nearly zero -- only the
  boxes break the symmetry -- so its own relative error is larger; printed);
* 384 x 384 x 192 dispersive grid (Drude + 2 Lorentz, TFSF, two 64-frequency
  planes): E and H, each taken as one vector, <= 1e-5, DFT <= 1e-4 per sampled
  frequency.  The cross-polarised components (Ey, Ez, Hx, Hz) of this x-polarised
  plane wave are small, so float32 rounding at the scale of Ex and Hy shows in
  their own relative errors (a few 1e-5); the per-component figures are printed;
* four seeded uneven couplers (seeds 0-3), 4000 steps, 64 frequencies:
  max |dS| <= 1e-3 per design.
"""

import glob
import json
import os

import numpy as np
import pytest

from oracle import fdtd64 as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def torch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _fixture(pattern):
    """The full-length fixture if present, else the longest snapshot."""
    paths = sorted(glob.glob(os.path.join(GOLDEN, pattern)))
    if not paths:
        pytest.skip(f"fixture {pattern} not generated")
    full = [p for p in paths if "_n" not in os.path.basename(p)]
    path = full[0] if full else paths[-1]
    z = np.load(path)
    return z, json.loads(str(z["meta"]))


def _compare_fields(got_fn, z, meta, tol=1e-5, vectors=False):
    """got_fn(c) -> float64 numpy component; compares full-field norms and the
    sampled planes per component, or (vectors) with E and H each as one vector."""
    from golden.make_config_fixtures import sample_fields

    got = sample_fields({c: got_fn(c) for c in O.COMPONENTS}, tuple(meta["dims"]))
    groups = [("E", ("Ex", "Ey", "Ez")), ("H", ("Hx", "Hy", "Hz"))] if vectors else [(c, (c,)) for c in O.COMPONENTS]
    errs = {}
    for name, comps in list(groups) + ([] if not vectors else [(c, (c,)) for c in O.COMPONENTS]):
        keys = [k for c in comps for k in z.files if k.startswith(f"pl_{c}_")]
        a = np.concatenate([got[k].ravel() for k in keys])
        b = np.concatenate([z[k].ravel() for k in keys])
        n_ref = float(np.sqrt(sum(float(z[f"norm_{c}"]) ** 2 for c in comps)))
        n_got = float(np.sqrt(sum(float(got[f"norm_{c}"]) ** 2 for c in comps)))
        errs[name] = {"planes": rel(a, b), "norm": abs(n_got - n_ref) / max(n_ref, 1e-300)}
    print("fp32 vs float64 oracle:", json.dumps(errs))
    for name, _ in groups:
        assert errs[name]["planes"] <= tol, (name, errs[name])
        assert errs[name]["norm"] <= tol, (name, errs[name])
    return errs


def test_3d_256_cpml_full_size_vs_oracle(torch):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.grid import YeeGrid
    from prismo_gb300.pml import PMLParams
    from prismo_gb300.sources import GaussianPulse
    from prismo_gb300.workloads import CONFIG_3D, boxes_3d

    z, meta = _fixture("oracle_c2_256*.npz")
    cfg = CONFIG_3D
    dims = tuple(meta["dims"])
    grid = YeeGrid.from_total(dims, cfg["dx"], cfg["cpml"])
    dt = grid.suggest_time_step(cfg["courant"])
    assert abs(dt - meta["dt"]) <= 1e-15 * dt
    n, every = meta["steps"], meta["trace_every"]
    wf = GaussianPulse(cfg["pulse_f0"], cfg["pulse_width"])
    c = tuple(d // 2 for d in dims)
    eng = FDTDEngine(grid.dimensions, grid.spacing, dt, is_2d=False, precision="fp32",
                     material_arrays={"eps_rel": boxes_3d(dims, seed=cfg["seed"])},
                     pml=PMLParams(thickness=cfg["cpml"]))
    eng.add_source("Ez", eng.offsets("Ez", tuple(np.array([v]).reshape(1, 1, 1) for v in c)), None, wf)
    amps = np.asarray(wf((np.arange(n) + 1) * dt), dtype=np.float64).reshape(n, 1)
    trace = []
    for s0 in range(0, n, every):  # the probe cells every `every` steps
        eng.step(every, amps[s0:s0 + every])
        ez = eng.component("Ez")  # a view of the current field set (the sets alternate)
        trace.append([float(ez[tuple(p)]) for p in meta["probes"]])
    assert eng.check_status() == 0
    want = z["trace_Ez"]
    got = np.array(trace)
    peak = np.abs(want).max(axis=0)
    terr = float((np.abs(got - want) / peak).max())
    print(f"probe traces: max |err| / peak = {terr:.2e} ({len(trace)} samples x {len(meta['probes'])} probes)")
    assert terr <= 1e-5
    _compare_fields(lambda comp: eng.component(comp).double().cpu().numpy(), z, meta, vectors=True)
    eng.close()


def test_dispersive_384_full_grid_vs_oracle(torch):
    from golden.make_config_fixtures import sample_dft
    from prismo_gb300.workloads import build_dispersive_engine

    z, meta = _fixture("oracle_c3_384_n*.npz")
    dims = tuple(meta["dims"])
    eng, info = build_dispersive_engine(dims, precision="fp32", cpml=meta["cpml"])
    assert abs(info["dt"] - meta["dt"]) <= 1e-15 * meta["dt"] and info["k_plane"] == meta["k_plane"]
    n = meta["steps"]
    t = (np.arange(n) + 1) * info["dt"]
    eng.step(n, info["waveform"](t)[:, None])
    assert eng.check_status() == 0
    print(f"dispersive grid {dims}, {n} steps")
    _compare_fields(lambda comp: eng.component(comp).double().cpu().numpy(), z, meta, vectors=True)
    nf = len(info["freqs"])
    for q, m in enumerate(info["dft_ids"]):
        d = eng.dft_result(m).cpu().numpy().reshape(nf, dims[0], dims[1] - 1)
        got = sample_dft(d)
        want = z[f"dft{q}_sample"]
        errs = [rel(got["sample"][f], want[f]) for f in range(want.shape[0])]
        nerr = np.abs(got["norm"] - z[f"dft{q}_norm"]) / np.maximum(z[f"dft{q}_norm"], 1e-300)
        print(f"DFT plane {q}: sampled rel L2 max {max(errs):.2e}, plane-norm rel max {nerr.max():.2e}")
        assert max(errs) <= 1e-4, (q, errs)
        assert nerr.max() <= 1e-4, (q, nerr.max())
    eng.close()


def test_dispersive_384_fp32_vs_fp64_full_length(torch):
    """The whole 4000-step dispersive run, float32 against the float64 kernels
    (which the test above and the reduced-size test pin to the oracle).  By step
    4000 the pulse has reflected off the metal and left through the CPML: the
    fields that remain are 3-20 % of their peak, so the error is measured against
    each field's peak norm over the run (E and H each as one vector, <= 1e-5); the
    DFT spectra, which integrate the whole run, against their own norms (<= 1e-4).
    The plain relative L2 of every component at step 4000 is printed as well."""
    from prismo_gb300.workloads import CONFIG_3D_DISPERSIVE, build_dispersive_engine

    n, chunk = CONFIG_3D_DISPERSIVE["steps"], 500
    engs = {p: build_dispersive_engine(precision=p) for p in ("fp64", "fp32")}
    info = engs["fp64"][1]
    peak = {"E": 0.0, "H": 0.0}
    vec = lambda e, g: torch.cat([e.component(c).double().flatten() for c in (g + "x", g + "y", g + "z")])  # noqa: E731
    for s0 in range(0, n, chunk):
        t = (np.arange(s0, s0 + chunk) + 1) * info["dt"]
        for eng, _ in engs.values():
            eng.step(chunk, info["waveform"](t)[:, None])
        for g in peak:
            peak[g] = max(peak[g], float(vec(engs["fp64"][0], g).norm()))
    e64, e32 = engs["fp64"][0], engs["fp32"][0]
    assert e64.check_status() == 0 and e32.check_status() == 0
    to_peak = {g: float((vec(e32, g) - vec(e64, g)).norm()) / peak[g] for g in peak}
    comp = {c: float((e32.component(c).double() - e64.component(c).double()).norm() / e64.component(c).double().norm())
            for c in O.COMPONENTS}
    print("dispersive, 4000 steps, fp32 vs fp64: error / peak norm", to_peak, "; per-component rel L2", comp)
    for g, e in to_peak.items():
        assert e <= 1e-5, (g, e)
    for q, m in enumerate(info["dft_ids"]):
        a, b = e32.dft_result(m).to(torch.complex128), e64.dft_result(m).to(torch.complex128)
        e = ((a - b).reshape(a.shape[0], -1).norm(dim=1) / b.reshape(b.shape[0], -1).norm(dim=1)).max().item()
        print(f"DFT plane {q}: max per-frequency rel L2 {e:.2e}")
        assert e <= 1e-4, (q, e)
    for eng, _ in engs.values():
        eng.close()


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_seeded_couplers_vs_oracle(torch, seed):
    from prismo_gb300 import sweep as S

    path = os.path.join(GOLDEN, f"oracle_c4_seed{seed:02d}.npz")
    if not os.path.exists(path):
        pytest.skip("fixture not generated")
    z = np.load(path)
    meta = json.loads(str(z["meta"]))
    d = S.coupler_design(seed)
    assert (d.nx, d.ny) == (meta["nx"], meta["ny"])
    r = S.batched_sweep([d], nsteps=meta["steps"], nfreq=meta["nfreq"])
    want = z["S"]
    err = float(np.abs(r.S[0] - want).max())
    print(f"coupler seed {seed} ({d.nx} x {d.ny}): max |S| {np.abs(want).max():.3f}, max |dS| {err:.2e}")
    assert err <= 1e-3, err
