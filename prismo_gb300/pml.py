"""CPML parameters and per-axis recursion coefficients.

``PMLParams`` mirrors boundaries/pml.py:23-46.  ``cpml_axis_coefficients``
computes, for one axis of ``n`` points, the arrays (b, a, kappa) that the
kernels index by each component's own index along that axis:

* profiles from ``CPML._compute_pml_parameters`` (boundaries/pml.py:117-151):
  rho = depth/t (depth 0..t-1), sigma = sigma_max rho^m,
  kappa = 1 + (kappa_max - 1) rho^m, alpha = alpha_max (1 - rho)^m,
  sigma_max defaulting to 0.8 (m+1) / (150 pi max(spacing));
* edge mapping from ``_compute_pml_coefficients`` (pml.py:219-250): the lower
  slab uses profile[t-1-i], the upper slab profile[i];
* the Roden-Gedney recursion b = exp(-(sigma/kappa + alpha) dt / eps0),
  a = sigma (b - 1) / (sigma kappa + kappa^2 alpha), with the simulation dt.
  (pml.py:196 uses suggest_time_step(0.9) and omits the 1/eps0, which leaves the
  layer transparent; both are corrected here.)
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

import numpy as np

EPS0 = 8.854187817e-12


@dataclass
class PMLParams:
    """boundaries/pml.py:23-46."""

    thickness: int
    sigma_max: Optional[float] = None
    kappa_max: float = 15.0
    alpha_max: float = 0.0
    polynomial_order: int = 3


def cpml_axis_coefficients(n: int, params: PMLParams, d_max: float, dt: float):
    t = int(params.thickness)
    b = np.ones(n)
    a = np.zeros(n)
    kap = np.ones(n)
    if t <= 0:
        return b, a, kap
    if 2 * t > n:
        raise ValueError(f"CPML thickness {t} does not fit an axis of {n} points")
    m = params.polynomial_order
    smax = params.sigma_max
    if smax is None:
        smax = 0.8 * (m + 1) / (150.0 * math.pi * d_max)
    rho = np.arange(t, dtype=np.float64) / t
    sigma = smax * rho**m
    kappa = 1.0 + (params.kappa_max - 1.0) * rho**m
    alpha = params.alpha_max * (1.0 - rho) ** m
    bb = np.exp(-(sigma / kappa + alpha) * dt / EPS0)
    with np.errstate(divide="ignore", invalid="ignore"):
        aa = np.where(sigma != 0, sigma / (sigma * kappa + kappa**2 * alpha) * (bb - 1.0), 0.0)
    b[:t] = bb[::-1]
    a[:t] = aa[::-1]
    kap[:t] = kappa[::-1]
    b[n - t:] = bb
    a[n - t:] = aa
    kap[n - t:] = kappa
    return b, a, kap
