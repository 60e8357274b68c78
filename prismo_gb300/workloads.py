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


def boxes_3d(dims, nboxes=32, seed=0, edge=(10, 80), eps_range=(1.0, EPS_SI), background=EPS_SIO2):
    """Dielectric of seeded axis-aligned boxes (3D FP32 plane configuration).

    Centres are uniform in the domain (cells), edges integer-uniform in
    ``edge`` cells per axis, permittivities uniform in ``eps_range``; painted in
    draw order.  Returns the cell-centred eps_rel array (nx, ny, nz), float64.
    """
    rng = np.random.default_rng(seed)
    nx, ny, nz = dims
    eps = np.full((nx, ny, nz), float(background))
    for _ in range(nboxes):
        c = rng.uniform(0.0, 1.0, size=3) * np.array([nx, ny, nz])
        e = rng.integers(edge[0], edge[1] + 1, size=3)
        v = rng.uniform(*eps_range)
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
