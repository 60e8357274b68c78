"""The 3D dispersive configuration (Drude + 2 Lorentz metal half-space, Si3N4
ridge, TFSF plane wave, two 64-frequency Ex DFT planes) at reduced size against
the float64 oracle: float32 fields rel L2 <= 1e-5, DFT planes <= 1e-4 per
frequency; float64 fields |err| <= 1e-11 x max.  Both schedules: the fused one
(TFSF corrections and the ADE partial update in the fused H + E kernel, the pole
terms in a pass over the metal) and the split kernels."""

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


@pytest.mark.parametrize("fused", [True, False])
def test_dispersive_config_reduced(torch, fused):
    from prismo_gb300.workloads import build_dispersive_engine

    dims, cpml, n = (40, 36, 64), 6, 700
    results = {}
    for prec in ("fp64", "fp32"):
        eng, info = build_dispersive_engine(dims, precision=prec, cpml=cpml, z_metal=24, ridge_width=0.3e-6)
        eng.set_fused_extras(fused)
        dt, wf = info["dt"], info["waveform"]
        t = (np.arange(n) + 1) * dt
        eng.step(n, wf(t)[:, None])
        assert eng.check_status() == 0
        results[prec] = ({c: eng.component(c).double().cpu().numpy() for c in O.COMPONENTS},
                         [eng.dft_result(m).cpu().numpy() for m in info["dft_ids"]])
        eng.close()
    g = O.OracleGrid.from_total(*dims, 20e-9, cpml)
    o = O.OracleFDTD(g, info["dt"], {"eps_rel": info["eps"]}, cpml_layers=cpml,
                     ade=[O.ADERegion(box=info["box"], eps_inf=1.0, poles=info["poles"])],
                     tfsf=O.TFSFPlane(k0=info["k_plane"], direction=-1, polarization="x", waveform=info["waveform"]))
    ids = [o.add_dft("Ex", p, info["freqs"]) for p in info["planes"]]
    o.run(n)
    assert np.abs(o.F["Ex"][:, :, : info["z_metal"]]).max() > 0  # the wave reached the metal
    f64, d64 = results["fp64"]
    f32, d32 = results["fp32"]
    for c in O.COMPONENTS:
        ref = o.F[c]
        np.testing.assert_allclose(f64[c], ref, rtol=0, atol=1e-11 * np.abs(ref).max(), err_msg=c)
        assert rel(f32[c], ref) <= 1e-5, (c, rel(f32[c], ref))
    for q, m in enumerate(ids):
        want = o.dfts[m].data.reshape(len(info["freqs"]), -1)
        for f in range(want.shape[0]):
            assert rel(d32[q][f], want[f]) <= 1e-4, (q, f, rel(d32[q][f], want[f]))


def test_fused_and_split_dispersive_schedules_agree(torch):
    """The two schedules on the same reduced configuration: float64 to 1e-12 of
    the field maxima; float32 (the curls' rounding differs) E and H, each as one
    vector, to 1e-6 rel L2 and every component to 1e-5 (the cross-polarised ones
    are small, so float32 rounding at the scale of Ex and Hy shows in their own
    relative errors)."""
    from prismo_gb300.workloads import build_dispersive_engine

    dims, cpml, n = (40, 36, 64), 6, 400
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
        out, spec, per_step = {}, {}, {}
        for fused in (True, False):
            eng, info = build_dispersive_engine(dims, precision=prec, cpml=cpml, z_metal=24, ridge_width=0.3e-6)
            eng.set_fused_extras(fused)
            t = (np.arange(n) + 1) * info["dt"]
            n0 = eng.launch_count()
            eng.step(n, info["waveform"](t)[:, None])
            per_step[fused] = (eng.launch_count() - n0) / n
            assert eng.check_status() == 0
            out[fused] = {c: eng.component(c).double().cpu().numpy() for c in O.COMPONENTS}
            spec[fused] = [eng.dft_result(m).cpu().numpy() for m in info["dft_ids"]]
            eng.close()
        # the DFT planes (one above the metal, one inside it) are sampled by the
        # fused kernel and the ADE pass on the fused schedule, by dft_sample on the
        # split one; float32: TFSF line + fused kernel + ADE pass per step, plus the
        # flushes every 16 steps
        print(f"{prec}: launches per step fused {per_step[True]:.2f}, split {per_step[False]:.2f}")
        if prec == "fp32":
            assert per_step[True] <= 3.3, per_step
        for q in range(len(spec[True])):
            a, b = spec[True][q], spec[False][q]
            e = np.linalg.norm(a - b) / np.linalg.norm(b)
            assert e <= (1e-12 if prec == "fp64" else 1e-5), (prec, q, e)
        for c in O.COMPONENTS:
            a, b = out[True][c], out[False][c]
            if prec == "fp64":
                np.testing.assert_allclose(a, b, rtol=0, atol=tol * np.abs(b).max(), err_msg=c)
            else:
                assert rel(a, b) <= 1e-5, (c, rel(a, b))
        if prec == "fp32":
            for g in ("E", "H"):
                a = np.concatenate([out[True][g + x].ravel() for x in "xyz"])
                b = np.concatenate([out[False][g + x].ravel() for x in "xyz"])
                print(f"fused vs split, float32, {g}: rel L2 {rel(a, b):.2e}")
                assert rel(a, b) <= tol, (g, rel(a, b))
