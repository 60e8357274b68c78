"""Seeded synthetic inputs for the benchmark configurations (host-side input prep).

Geometry is rasterised with the reference's point-sampling rule:
``Box.contains`` tests |p - centre| <= size/2 on every axis at cell centres
(geometry/shapes.py:71-132); later boxes overwrite earlier ones.
"""

from __future__ import annotations

import numpy as np

C0 = 299792458.0

EPS_SI = 12.11
EPS_SIO2 = 2.085


def _axis_mask(n: int, centre: float, size: float) -> np.ndarray:
    pts = np.arange(n) + 0.5
    return np.abs(pts - centre) <= size / 2.0


def box_specs_3d(dims, nboxes=32, seed=0, edge=(10, 80), eps_range=(1.0, EPS_SI)):
    """The seeded boxes of the 3D FP32 plane configuration, in draw order:
    (centre, edges, eps) with the centre uniform in the domain and the edges
    integer-uniform in ``edge``, both in cells; eps uniform in ``eps_range``."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nboxes):
        c = rng.uniform(0.0, 1.0, size=3) * np.array(dims, dtype=np.float64)
        e = rng.integers(edge[0], edge[1] + 1, size=3)
        v = rng.uniform(*eps_range)
        out.append((c, e, v))
    return out


def boxes_3d(dims, nboxes=32, seed=0, edge=(10, 80), eps_range=(1.0, EPS_SI), background=EPS_SIO2):
    """Dielectric of seeded axis-aligned boxes (3D FP32 plane configuration).

    Boxes from ``box_specs_3d``, painted in draw order (later boxes win) by the
    point-sampling rule at cell centres.  Returns the cell-centred eps_rel array
    (nx, ny, nz), float64.
    """
    nx, ny, nz = dims
    eps = np.full((nx, ny, nz), float(background))
    for c, e, v in box_specs_3d(dims, nboxes, seed, edge, eps_range):
        mx = _axis_mask(nx, c[0], e[0])
        my = _axis_mask(ny, c[1], e[1])
        mz = _axis_mask(nz, c[2], e[2])
        m = mx[:, None, None] & my[None, :, None] & mz[None, None, :]
        eps[m] = v
    return eps


def slab_waveguide_2d(dims, dx, width=0.5e-6, eps_core=EPS_SI, eps_clad=EPS_SIO2):
    """2D straight slab waveguide along x, centred in y (2D TE drop-in configuration)."""
    nx, ny = dims[0], dims[1]
    eps = np.full((nx, ny, 1), float(eps_clad))
    my = _axis_mask(ny, ny / 2.0, width / dx)
    eps[:, my, 0] = eps_core
    return eps


def wavelengths_to_freqs(lmin, lmax, n):
    lam = np.linspace(lmin, lmax, n)
    return C0 / lam


# -- the 3D FP32 plane configuration: 256^3, 12-cell CPML, 2000 steps ---------------
CONFIG_3D = {
    "name": "3d_fp32_cpml_256",
    "dims": (256, 256, 256),
    "dx": 20e-9,
    "cpml": 12,
    "steps": 2000,
    "courant": 0.5,
    "nboxes": 32,
    "seed": 0,
    "pulse_f0": 193e12,
    "pulse_width": 10e-15,
}


def config_3d_inputs(dims=None, seed=0):
    cfg = dict(CONFIG_3D)
    if dims is not None:
        cfg["dims"] = tuple(dims)
    eps = boxes_3d(cfg["dims"], nboxes=cfg["nboxes"], seed=seed)
    return cfg, eps


# -- the 2D TE drop-in configuration: 500x250 total, 20-cell CPML, 3000 steps --------
CONFIG_2D = {
    "name": "2d_te_waveguide_500x250",
    "dims": (500, 250, 1),
    "dx": 20e-9,
    "cpml": 20,
    "steps": 3000,
    "courant": 0.5,
    "pulse_f0": 193e12,
    "pulse_width": 10e-15,
    "nfreq": 11,
}


def config_2d_layout(dims=(500, 250, 1), cpml=20, dx=20e-9):
    """Slab waveguide along x (Si 0.5 um in SiO2); soft Ez line source across the
    slab at x = cpml + 10, DFT line (all y) at x = nx - cpml - 10, 11 frequencies
    for wavelengths 1.5-1.6 um.  Index sets are in Ez's own indices."""
    nx, ny = dims[0], dims[1]
    eps = slab_waveguide_2d(dims, dx)
    core = np.nonzero(_axis_mask(ny, ny / 2.0, 0.5e-6 / dx))[0]
    src = (np.array([cpml + 10]).reshape(1, 1), core.reshape(1, -1))
    mon = (np.array([nx - cpml - 10]).reshape(1, 1), np.arange(ny - 1).reshape(1, -1))
    freqs = wavelengths_to_freqs(1.5e-6, 1.6e-6, 11)
    return eps, src, mon, freqs


# -- the 3D dispersive configuration: 384x384x192, Drude-Lorentz metal, TFSF ----------
CONFIG_3D_DISPERSIVE = {
    "name": "3d_dispersive_384x384x192",
    "dims": (384, 384, 192),
    "dx": 20e-9,
    "cpml": 12,
    "steps": 4000,
    "z_metal": 96,
    "ridge_width": 1.0e-6,
    "ridge_height": 0.4e-6,
    "eps_ridge": 4.0,
    "omega_p": 1.37e16,
    "gamma_d": 1.0e14,
    "nfreq": 64,
}


def config_3d_dispersive(dims=(384, 384, 192), seed=0, dx=20e-9, z_metal=None):
    """Half-space Drude + 2-Lorentz metal (z < z_metal, eps_inf = 1), a Si3N4 ridge
    (eps 4.0, 1 um wide along y, 0.4 um high) on it, air above; seeded Lorentz
    poles (omega0 U[3e15, 6e15], delta_eps U[0.5, 2], gamma U[1e14, 5e14]).
    Returns eps (cell-centred), the metal box (E indices), the pole list
    (materials.LorentzPole) and the TFSF plane index (above the ridge, -z)."""
    from .materials import LorentzPole

    rng = np.random.default_rng(seed)
    nx, ny, nz = dims
    zm = z_metal if z_metal is not None else nz // 2
    eps = np.ones(dims)
    ridge_h = int(round(0.4e-6 / dx))
    my = _axis_mask(ny, ny / 2.0, 1.0e-6 / dx)
    eps[:, my, zm:zm + ridge_h] = 4.0
    lor = [LorentzPole(omega_0=rng.uniform(3e15, 6e15), delta_epsilon=rng.uniform(0.5, 2.0),
                       gamma=rng.uniform(1e14, 5e14)) for _ in range(2)]
    box = (0, nx, 0, ny, 0, zm)
    k_plane = min(nz - 12 - 8, zm + ridge_h + (nz - zm - ridge_h) // 2)
    return eps, box, lor, k_plane


def dispersive_monitor_planes(dims, z_metal, ridge_h, k_plane):
    """Ex DFT planes (Ex indices, all x and y): halfway between the ridge top and
    the TFSF plane, and 2 cells inside the metal."""
    nx, ny, nz = dims
    k_up = (z_metal + ridge_h + k_plane) // 2
    k_dn = max(1, z_metal - 2)
    idx = lambda k: (np.arange(nx)[:, None, None], np.arange(ny - 1)[None, :, None], np.array([[[k]]]))  # noqa: E731
    return [idx(k_up), idx(k_dn)]


def build_dispersive_engine(dims=(384, 384, 192), precision="fp32", cpml=12, dx=20e-9, nfreq=64, seed=0,
                            z_metal=None, ridge_width=1.0e-6, device=None):
    """The 3D dispersive configuration on the device engine: Drude + 2 Lorentz
    half-space metal (eps_inf 1) under a Si3N4 ridge, Ex-polarised plane wave
    injected by a TFSF plane above the ridge travelling towards the metal (-z),
    and two 64-frequency Ex DFT planes (1.5-1.6 um).  Returns (engine, info)
    with info holding dt, eps, the metal box, the pole dicts, the TFSF plane,
    the waveform and the monitor index sets."""
    from .engine import FDTDEngine
    from .materials import DrudeLorentzMaterial
    from .pml import PMLParams
    from .sources import GaussianPulse

    nx, ny, nz = dims
    zm = z_metal if z_metal is not None else nz // 2
    eps, box, lor, k_plane = config_3d_dispersive(dims, seed=seed, dx=dx, z_metal=zm)
    if ridge_width != 1.0e-6:  # reduced grids: narrower ridge
        eps = np.ones(dims)
        ridge_h = int(round(0.4e-6 / dx))
        my = _axis_mask(ny, ny / 2.0, ridge_width / dx)
        eps[:, my, zm:zm + ridge_h] = 4.0
    ridge_h = int(round(0.4e-6 / dx))
    k_plane = min(nz - cpml - 8, zm + ridge_h + (nz - zm - ridge_h) // 2)
    dt = 0.5 / (C0 * np.sqrt(3.0 / dx**2))
    metal = DrudeLorentzMaterial(1.0, 1.37e16, 1.0e14, lor)
    poles = metal.ade_poles(dt)
    wf = GaussianPulse(193e12, 10e-15)
    eng = FDTDEngine(dims, (dx, dx, dx), dt, is_2d=False, precision=precision, material_arrays={"eps_rel": eps},
                     pml=PMLParams(thickness=cpml), device=device)
    eng.set_dispersive([(box, 1.0, poles)])
    eng.set_tfsf(k_plane, -1, "x", wf)
    planes = dispersive_monitor_planes(dims, zm, ridge_h, k_plane)
    freqs = wavelengths_to_freqs(1.5e-6, 1.6e-6, nfreq)
    mids = [eng.add_dft("Ex", eng.offsets("Ex", p), freqs, t0=dt) for p in planes]
    info = dict(dt=dt, eps=eps, box=box, poles=poles, k_plane=k_plane, waveform=wf, planes=planes, freqs=freqs,
                dft_ids=mids, z_metal=zm, ridge_h=ridge_h)
    return eng, info


def dispersive_bytes_per_cell(dims, cpml, box, npoles_lorentz, nplanes, nfreq, model="per_step"):
    """Algorithmic float32 bytes per cell update of the dispersive configuration:
    6 fields R+W and 3 Cb (60 B), CPML psi on the slabs (32 B x slab fraction per
    axis), the ADE auxiliaries on metal cells (Drude J read and written: 3 x 8 B;
    each Lorentz pole's P and increment D read and written: 3 x 16 B) and the
    DFT on the monitor planes
    (sampled Ex).  ``model="per_step"``: the running sums (re, im and their Kahan
    compensations, 16 B read + 16 B written per frequency) updated every step;
    ``model="ring"``: as this implementation does it, the samples written to a
    16-step ring (4 B) and read back at the flush (4 B), the sums touched once
    per 16 steps."""
    nx, ny, nz = dims
    n = nx * ny * nz
    b = 60.0 + 32.0 * sum(2.0 * cpml / m for m in dims)
    metal = (box[1] - box[0]) * (box[3] - box[2]) * (box[5] - box[4]) / n
    b += metal * (3 * 8 + npoles_lorentz * 3 * 16)
    plane = nplanes * nx * ny / n
    if model == "per_step":
        b += plane * nfreq * 32
    elif model == "ring":
        b += plane * (nfreq * 32 / 16.0 + 8.0)
    else:
        raise ValueError(model)
    return b
