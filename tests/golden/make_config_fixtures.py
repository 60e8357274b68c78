"""Float64-oracle fixtures for the benchmark configurations at their real sizes.

TEST INFRASTRUCTURE: runs ``oracle/fdtd64.py`` (the NumPy float64 restatement of
the reference stepper) on the CPU and stores compact fixtures that the ``-m gpu``
tests compare the device kernels against.  The full fields are far too large to
commit, so each fixture keeps

* per component: the full-field L2 norm and sum, and every 4th cell of three
  planes normal to each axis (nine planes per component);
* time traces of a few probe cells (configuration 2);
* DFT planes: per-frequency full-plane L2 norms and sums, and every 8th point of
  every 8th frequency (configuration 3);
* complex S-parameters for 64 frequencies (configuration 4).

Usage (one job per process; they run for hours on one core each)::

    python tests/golden/make_config_fixtures.py c2             # 256^3, 2000 steps
    python tests/golden/make_config_fixtures.py c3 [steps]     # 384x384x192
    python tests/golden/make_config_fixtures.py c4 SEED [...]  # seeded couplers

Fixtures are written next to this script; configurations 2 and 3 also write
intermediate snapshots (``..._nNNNN.npz``) so that a run cut short still leaves
a usable fixture.
"""

from __future__ import annotations

import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import fdtd64 as O  # noqa: E402

STRIDE = 4


def plane_positions(dims):
    """Three plane indices per axis: near the low CPML edge, the centre, and
    three quarters of the way up."""
    return [(8, n // 2, (3 * n) // 4) for n in dims]


def sample_fields(F, dims):
    """Compact record of the six field components (see the module docstring)."""
    out = {}
    pos = plane_positions(dims)
    for c in O.COMPONENTS:
        a = F[c]
        out[f"norm_{c}"] = np.array(np.linalg.norm(a))
        out[f"sum_{c}"] = np.array(a.sum())
        for ax in range(3):
            for q, p in enumerate(pos[ax]):
                sl = [slice(None, None, STRIDE)] * 3
                sl[ax] = min(p, a.shape[ax] - 1)
                out[f"pl_{c}_{ax}_{q}"] = np.ascontiguousarray(a[tuple(sl)])
    return out


def sample_field_gpu(get, dims):
    """The same record from device components (``get(c)`` returns a float64
    numpy array of component ``c``).  Used by the GPU tests."""
    return sample_fields({c: get(c) for c in O.COMPONENTS}, dims)


DFT_F_STRIDE = 8
DFT_P_STRIDE = 8


def sample_dft(data):
    """``data``: (nfreq, nx, ny) complex plane spectra."""
    return {
        "norm": np.linalg.norm(data.reshape(data.shape[0], -1), axis=1),
        "sum": data.reshape(data.shape[0], -1).sum(axis=1),
        "sample": np.ascontiguousarray(data[::DFT_F_STRIDE, ::DFT_P_STRIDE, ::DFT_P_STRIDE]),
    }


def _save(path, meta, arrays):
    np.savez_compressed(path, meta=json.dumps(meta), **arrays)
    print("wrote", path, flush=True)


# -- configuration 2: 256^3 FP32 CPML, 32 seeded boxes, Ez dipole, 2000 steps ----------
C2_PROBES = [(128, 128, 128), (128, 128, 160), (100, 140, 128), (60, 200, 90), (200, 40, 210)]
C2_TRACE_EVERY = 50


def config2(steps=2000, snapshots=(500, 1000)):
    from prismo_gb300.workloads import CONFIG_3D, boxes_3d

    cfg = CONFIG_3D
    dims = cfg["dims"]
    g = O.OracleGrid.from_total(*dims, cfg["dx"], cfg["cpml"])
    dt = g.suggest_dt(cfg["courant"])
    eps = boxes_3d(dims, nboxes=cfg["nboxes"], seed=cfg["seed"])
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=cfg["cpml"])
    c = tuple(d // 2 for d in dims)
    o.add_source("Ez", tuple(np.array([v]).reshape(1, 1, 1) for v in c), O.gaussian_pulse(cfg["pulse_f0"],
                                                                                        cfg["pulse_width"]))
    trace = []
    meta = dict(config="3d_fp32_cpml_256", dims=dims, dx=cfg["dx"], cpml=cfg["cpml"], courant=cfg["courant"],
                seed=cfg["seed"], dt=dt, probes=C2_PROBES, trace_every=C2_TRACE_EVERY, stride=STRIDE,
                planes=plane_positions(dims))
    t0 = time.time()
    for n in range(1, steps + 1):
        o.step()
        if n % C2_TRACE_EVERY == 0:
            trace.append([o.F["Ez"][p] for p in C2_PROBES])
            print(f"c2 step {n} {time.time() - t0:.0f}s", flush=True)
        if n in snapshots or n == steps:
            m = dict(meta, steps=n)
            arr = sample_fields(o.F, dims)
            arr["trace_Ez"] = np.array(trace)
            name = "oracle_c2_256.npz" if n == steps else f"oracle_c2_256_n{n:04d}.npz"
            _save(os.path.join(HERE, name), m, arr)


# -- configuration 3: 384x384x192 dispersive, TFSF, two 64-frequency Ex planes ----------
def config3(steps=1000, snapshots=(300, 600, 1000, 1500)):
    from prismo_gb300.materials import DrudeLorentzMaterial
    from prismo_gb300.workloads import (CONFIG_3D_DISPERSIVE, config_3d_dispersive, dispersive_monitor_planes,
                                        wavelengths_to_freqs)

    cfg = CONFIG_3D_DISPERSIVE
    dims, dx, cpml = cfg["dims"], cfg["dx"], cfg["cpml"]
    zm = dims[2] // 2
    eps, box, lor, _ = config_3d_dispersive(dims, seed=0, dx=dx, z_metal=zm)
    ridge_h = int(round(0.4e-6 / dx))
    k_plane = min(dims[2] - cpml - 8, zm + ridge_h + (dims[2] - zm - ridge_h) // 2)
    dt = 0.5 / (O.C0 * np.sqrt(3.0 / dx**2))
    poles = DrudeLorentzMaterial(1.0, cfg["omega_p"], cfg["gamma_d"], lor).ade_poles(dt)
    g = O.OracleGrid.from_total(*dims, dx, cpml)
    wf = O.gaussian_pulse(193e12, 10e-15)
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=cpml,
                     ade=[O.ADERegion(box=box, eps_inf=1.0, poles=poles)],
                     tfsf=O.TFSFPlane(k0=k_plane, direction=-1, polarization="x", waveform=wf))
    freqs = wavelengths_to_freqs(1.5e-6, 1.6e-6, cfg["nfreq"])
    ids = [o.add_dft("Ex", p, freqs) for p in dispersive_monitor_planes(dims, zm, ridge_h, k_plane)]
    meta = dict(config="3d_dispersive_384x384x192", dims=dims, dx=dx, cpml=cpml, dt=dt, z_metal=zm,
                k_plane=k_plane, stride=STRIDE, planes=plane_positions(dims), dft_f_stride=DFT_F_STRIDE,
                dft_p_stride=DFT_P_STRIDE)
    t0 = time.time()
    for n in range(1, steps + 1):
        o.step()
        if n % 25 == 0:
            print(f"c3 step {n} {time.time() - t0:.0f}s", flush=True)
        if n in snapshots or n == steps:
            arr = sample_fields(o.F, dims)
            for q, m in enumerate(ids):
                d = o.dfts[m].data.reshape(len(freqs), dims[0], dims[1] - 1)
                for k, v in sample_dft(d).items():
                    arr[f"dft{q}_{k}"] = v
            _save(os.path.join(HERE, f"oracle_c3_384_n{n:04d}.npz"), dict(meta, steps=n), arr)


# -- configuration 4: seeded uneven couplers, 4000 steps, 64 frequencies ---------------
def oracle_s(layout, nsteps, freqs, dt):
    """S-parameters of one coupler from two oracle runs (the coupler and its
    straight normalisation guide), combined by ``sweep.s_parameters``."""
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


def config4(seed):
    from prismo_gb300 import sweep as S

    d = S.coupler_design(seed)
    L = S.coupler_layout(d)
    freqs = S.sweep_freqs(S.NFREQ)
    t0 = time.time()
    s = oracle_s(L, S.STEPS, freqs, S.sweep_dt())
    print(f"c4 seed {seed} {time.time() - t0:.0f}s", flush=True)
    meta = dict(config="coupler_sweep", seed=seed, nx=d.nx, ny=d.ny, width=d.width, gap=d.gap, length=d.length,
                steps=S.STEPS, nfreq=S.NFREQ)
    _save(os.path.join(HERE, f"oracle_c4_seed{seed:02d}.npz"), meta, {"S": s, "freqs": freqs})


if __name__ == "__main__":
    job = sys.argv[1]
    if job == "c2":
        config2()
    elif job == "c3":
        config3(int(sys.argv[2]) if len(sys.argv) > 2 else 1000)
    elif job == "c4":
        for s in sys.argv[2:]:
            config4(int(s))
    else:
        raise SystemExit(__doc__)
