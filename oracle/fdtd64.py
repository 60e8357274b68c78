"""NumPy float64 restatement of the reference FDTD stepper -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline legs
use this module; it is the checker, never the product path.

Every function cites the reference file (paths inside the Prismo project) whose
arithmetic it restates.  Arrays use the reference layout: C order, component
shapes from ``core/grid.py:137-176`` (z fastest).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

# Physical constants exactly as the reference spells them
# (core/solver.py:63-65, boundaries/pml.py:89-90, materials/ade.py:69).
EPS0 = 8.854187817e-12
MU0 = 4 * np.pi * 1e-7
C0 = 299792458.0

COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


# ----------------------------------------------------------------------------
# Grid semantics (core/grid.py)
# ----------------------------------------------------------------------------
class OracleGrid:
    """Restates ``YeeGrid`` (core/grid.py:53-176, 258-354, 383-513)."""

    def __init__(self, size, resolution, boundary_layers: int = 10):
        if isinstance(resolution, (int, float)):
            resolution = (resolution, resolution, resolution)
        self.Lx, self.Ly, self.Lz = size
        self.res = tuple(float(r) for r in resolution)
        self.dx = 1.0 / self.res[0]
        self.dy = 1.0 / self.res[1]
        self.dz = 1.0 / self.res[2]
        self.is_2d = self.Lz == 0.0
        # core/grid.py:96-100 -- ceil of physical size times resolution
        self.Nx = int(np.ceil(self.Lx * self.res[0])) if self.Lx > 0 else 1
        self.Ny = int(np.ceil(self.Ly * self.res[1])) if self.Ly > 0 else 1
        self.Nz = int(np.ceil(self.Lz * self.res[2])) if self.Lz > 0 else 1
        if self.is_2d:
            self.Nz = 1
            self.dz = 0.0
        t = boundary_layers
        self.pml_layers = t
        # core/grid.py:107-111 -- boundary layers are added outside
        self.nx = self.Nx + 2 * t
        self.ny = self.Ny + 2 * t
        self.nz = self.Nz + (0 if self.is_2d else 2 * t)
        self.origin = np.array([-t * self.dx, -t * self.dy, 0.0 if self.is_2d else -t * self.dz])

    @classmethod
    def from_total(cls, nx: int, ny: int, nz: int, d: float, layers: int) -> "OracleGrid":
        """Grid whose *total* size (boundary layers included) is nx x ny x nz.

        The physical size is set half a cell short of the integer so that the
        reference's ``ceil`` lands exactly on ``n - 2*layers``.
        """
        if nz <= 1:
            size = ((nx - 2 * layers - 0.5) * d, (ny - 2 * layers - 0.5) * d, 0.0)
        else:
            size = ((nx - 2 * layers - 0.5) * d, (ny - 2 * layers - 0.5) * d, (nz - 2 * layers - 0.5) * d)
        g = cls(size, 1.0 / d, layers)
        assert g.dims == (nx, ny, max(nz, 1)), (g.dims, (nx, ny, nz))
        return g

    @property
    def dims(self):
        return (self.nx, self.ny, self.nz)

    @property
    def spacing(self):
        return (self.dx, self.dy, self.dz)

    def shape(self, comp: str):
        """core/grid.py:157-168."""
        nx, ny, nz = self.dims
        s3 = {
            "Ex": (nx, ny - 1, nz - 1),
            "Ey": (nx - 1, ny, nz - 1),
            "Ez": (nx - 1, ny - 1, nz),
            "Hx": (nx - 1, ny, nz),
            "Hy": (nx, ny - 1, nz),
            "Hz": (nx, ny, nz - 1),
        }
        s2 = {
            "Ex": (nx, ny - 1),
            "Ey": (nx - 1, ny),
            "Ez": (nx - 1, ny - 1),
            "Hx": (nx - 1, ny),
            "Hy": (nx, ny - 1),
            "Hz": (nx, ny),
        }
        return (s2 if self.is_2d else s3)[comp]

    def courant(self, dt: float) -> float:
        """core/grid.py:258-288."""
        inv = (1 / self.dx) ** 2 + (1 / self.dy) ** 2
        if not self.is_2d:
            inv += (1 / self.dz) ** 2
        return C0 * dt * np.sqrt(inv)

    def suggest_dt(self, safety_factor: float = 0.9) -> float:
        """core/grid.py:304-326."""
        inv = (1 / self.dx) ** 2 + (1 / self.dy) ** 2
        if not self.is_2d:
            inv += (1 / self.dz) ** 2
        return safety_factor / (C0 * np.sqrt(inv))

    def point_to_index(self, point):
        """core/grid.py:328-354 (clamps to the *physical* count, a reference quirk)."""
        x, y, z = point
        i = int(round((x - self.origin[0]) / self.dx))
        j = int(round((y - self.origin[1]) / self.dy))
        k = int(round((z - self.origin[2]) / self.dz)) if not self.is_2d else 0
        i = max(0, min(i, self.Nx - 1))
        j = max(0, min(j, self.Ny - 1))
        k = max(0, min(k, self.Nz - 1))
        return (i, j, k)

    def component_indices(self, comp, x_min, x_max, y_min, y_max, z_min, z_max):
        """core/grid.py:383-513 -- ``np.ix_`` index tuple of a region."""
        x_min = max(0, min(x_min, self.Nx - 1))
        x_max = max(1, min(x_max, self.Nx))
        y_min = max(0, min(y_min, self.Ny - 1))
        y_max = max(1, min(y_max, self.Ny))
        if not self.is_2d:
            z_min = max(0, min(z_min, self.Nz - 1))
            z_max = max(1, min(z_max, self.Nz))
        else:
            z_min, z_max = 0, 1
        shp = self.shape(comp)
        xr = range(x_min, min(x_max, shp[0]))
        yr = range(y_min, min(y_max, shp[1]))
        if self.is_2d:
            return np.ix_(xr, yr)
        zr = range(z_min, min(z_max, shp[2]))
        return np.ix_(xr, yr, zr)

    def region_bounds(self, center, size):
        """sources/base.py:97-139 and monitors/base.py:92-134 (identical)."""
        h = [s / 2 for s in size]
        lo = self.point_to_index((center[0] - h[0], center[1] - h[1], center[2] - h[2]))
        hi = self.point_to_index((center[0] + h[0], center[1] + h[1], center[2] + h[2]))
        x0, y0, z0 = lo
        x1, y1, z1 = hi
        if x0 == x1:
            x1 = x0 + 1
        if y0 == y1:
            y1 = y0 + 1
        if z0 == z1 and not self.is_2d:
            z1 = z0 + 1
        return x0, x1, y0, y1, z0, z1


# ----------------------------------------------------------------------------
# Waveforms (sources/waveform.py)
# ----------------------------------------------------------------------------
def gaussian_pulse(frequency, pulse_width, amplitude=1.0, phase=0.0, delay=None) -> Callable:
    """sources/waveform.py:107-152 -- A exp(-tau^2/2) sin(w t + phi), tau=(t-delay)/width."""
    omega = 2 * np.pi * frequency
    d = delay if delay is not None else 3 * pulse_width

    def f(t):
        tau = (t - d) / pulse_width
        return amplitude * np.exp(-0.5 * tau * tau) * np.sin(omega * t + phase)

    return f


def continuous_wave(frequency, amplitude=1.0, phase=0.0) -> Callable:
    """sources/waveform.py:63-96."""
    omega = 2 * np.pi * frequency
    return lambda t: amplitude * np.sin(omega * t + phase)


# ----------------------------------------------------------------------------
# CPML coefficients (boundaries/pml.py)
# ----------------------------------------------------------------------------
def cpml_profile(n: int, t: int, d_max: float, dt: float, m: int = 3, kappa_max: float = 15.0,
                 alpha_max: float = 0.0, sigma_max: Optional[float] = None, eps0_scaled: bool = True):
    """Per-index CPML arrays (b, a, kappa) of length ``n`` along one axis.

    Profiles follow ``CPML._compute_pml_parameters`` (boundaries/pml.py:117-151):
    rho = depth/t with depth = 0..t-1, sigma = sigma_max rho^m,
    kappa = 1 + (kappa_max-1) rho^m, alpha = alpha_max (1-rho)^m, and the default
    sigma_max = 0.8 (m+1) / (150 pi max(d)).  The index mapping follows
    ``_compute_pml_coefficients`` (pml.py:184-257): the lower edge uses
    profile[t-1-i], the upper edge profile[i].

    Two deliberate differences from pml.py, both required for a working CPML:
    the simulation ``dt`` is used (pml.py:196 takes ``suggest_time_step(0.9)``),
    and the exponent carries the 1/eps0 of the Roden-Gedney recursion,
    b = exp(-(sigma/kappa + alpha) dt/eps0), a = sigma (b-1) / (sigma kappa + kappa^2 alpha).
    ``eps0_scaled=False`` reproduces pml.py's unscaled exponent, for pinning.
    """
    b = np.ones(n)
    a = np.zeros(n)
    kap = np.ones(n)
    if t <= 0:
        return b, a, kap
    if sigma_max is None:
        sigma_max = 0.8 * (m + 1) / (150.0 * np.pi * d_max)
    depth = np.arange(t, dtype=np.float64)
    rho = depth / t
    sigma = sigma_max * rho**m
    kappa = 1.0 + (kappa_max - 1.0) * rho**m
    alpha = alpha_max * (1.0 - rho) ** m

    def coeff(idx):
        scale = dt / EPS0 if eps0_scaled else dt
        bb = np.exp(-(sigma[idx] / kappa[idx] + alpha[idx]) * scale)
        aa = 0.0
        if sigma[idx] != 0:
            aa = sigma[idx] / (sigma[idx] * kappa[idx] + kappa[idx] ** 2 * alpha[idx]) * (bb - 1.0)
        return bb, aa, kappa[idx]

    for i in range(t):
        b[i], a[i], kap[i] = coeff(t - 1 - i)
        b[n - t + i], a[n - t + i], kap[n - t + i] = coeff(i)
    return b, a, kap


# ----------------------------------------------------------------------------
# ADE coefficients (materials/dispersion.py)
# ----------------------------------------------------------------------------
def lorentz_coeffs(delta_eps, omega0, gamma, dt):
    """materials/dispersion.py:189-231 (bilinear C0..C3; C1 = C0)."""
    denom = 4.0 + 2 * gamma * dt + omega0**2 * dt**2
    c0 = 2 * delta_eps * omega0**2 * dt**2 / denom
    c2 = (8.0 - 2 * omega0**2 * dt**2) / denom
    c3 = -(4.0 - 2 * gamma * dt + omega0**2 * dt**2) / denom
    return {"kind": "lorentz", "C0": c0, "C1": c0, "C2": c2, "C3": c3}


def drude_coeffs(omega_p, gamma, dt):
    """materials/dispersion.py:267-286 (exponential step)."""
    e = np.exp(-gamma * dt)
    return {"kind": "drude", "C0": omega_p**2 / gamma * (1.0 - e), "C1": e}


def debye_coeffs(eps_s, eps_inf, tau, dt):
    """materials/dispersion.py:323-336."""
    e = np.exp(-dt / tau)
    return {"kind": "debye", "C0": (eps_s - eps_inf) * (1.0 - e), "C1": e}


def ade_e_coefficients(eps_inf: float, poles: Sequence[dict], dt: float):
    """Coefficients of the ADE-coupled E update used by both oracle and kernels.

    The reference updates P/J but never couples them to E (materials/ade.py:291-331).
    Coupling used here (P and J normalised by eps0, S = (dt/eps0) curl H):

    * Lorentz: P+ = C0 E+ + C1 E + C2 P + C3 P-      (ade.py:116-138 with E^n for C1)
      eps_inf (E+ - E) + (P+ - P) = S
    * Drude:   J+ = C1 J + C0 (E+ + E)/2              (ade.py:140-149, E time-centred)
      eps_inf (E+ - E) = S - dt (J+ + J)/2
    * Debye:   P+ = C1 P + C0 (E+ + E)/2              (ade.py:151-160, E time-centred)
      eps_inf (E+ - E) + (P+ - P) = S

    Solved for E+:  E+ = (ce*E + S - sum_p aux_p) / den, returned as
    (ce/den, 1/den) plus per-pole history weights.
    """
    den = eps_inf
    ce = eps_inf
    for p in poles:
        if p["kind"] == "lorentz":
            den += p["C0"]
            ce -= p["C1"]
        elif p["kind"] == "drude":
            den += dt * p["C0"] / 4.0
            ce -= dt * p["C0"] / 4.0
        elif p["kind"] == "debye":
            den += p["C0"] / 2.0
            ce -= p["C0"] / 2.0
        else:
            raise ValueError(p["kind"])
    return ce / den, 1.0 / den


# ----------------------------------------------------------------------------
# Reference coefficient interpolation (core/solver.py:458-533)
# ----------------------------------------------------------------------------
def _interp3(comp, a):
    if comp == "Ex":
        return 0.25 * (a[:, :-1, :-1] + a[:, 1:, :-1] + a[:, :-1, 1:] + a[:, 1:, 1:])
    if comp == "Ey":
        return 0.25 * (a[:-1, :, :-1] + a[1:, :, :-1] + a[:-1, :, 1:] + a[1:, :, 1:])
    if comp == "Ez":
        return 0.25 * (a[:-1, :-1, :] + a[1:, :-1, :] + a[:-1, 1:, :] + a[1:, 1:, :])
    if comp == "Hx":
        return 0.5 * (a[:-1, :, :] + a[1:, :, :])
    if comp == "Hy":
        return 0.5 * (a[:, :-1, :] + a[:, 1:, :])
    if comp == "Hz":
        return 0.5 * (a[:, :, :-1] + a[:, :, 1:])
    raise ValueError(comp)


def _interp2(comp, a):
    if comp == "Ex":
        return 0.5 * (a[:, :-1] + a[:, 1:])
    if comp == "Ey":
        return 0.5 * (a[:-1, :] + a[1:, :])
    if comp == "Ez":
        return 0.25 * (a[:-1, :-1] + a[1:, :-1] + a[:-1, 1:] + a[1:, 1:])
    if comp == "Hz":
        return a
    if comp == "Hx":
        return 0.5 * (a[:-1, :] + a[1:, :])
    if comp == "Hy":
        return 0.5 * (a[:, :-1] + a[:, 1:])
    raise ValueError(comp)


@dataclass
class ADERegion:
    """A dispersive box in E-index space with its material (ade.py:262-289)."""
    box: tuple  # (x0, x1, y0, y1, z0, z1) in each E component's own indices
    eps_inf: float
    poles: list  # dicts from lorentz_coeffs / drude_coeffs / debye_coeffs


@dataclass
class TFSFPlane:
    """Plane-wave injection on a z-plane fed by a 1D auxiliary grid (3D only)."""
    k0: int
    direction: int  # +1 or -1 (propagation along +z or -z)
    polarization: str  # "x" or "y"
    waveform: Callable
    eps_b: float = 1.0
    m0: int = 4
    max_steps: int = 20000


@dataclass
class _Source:
    comp: str
    index: tuple
    weight: object
    waveform: Callable


@dataclass
class _DFT:
    comp: str
    index: tuple
    freqs: np.ndarray
    data: np.ndarray = field(default=None)


class OracleFDTD:
    """FP64 FDTD stepper restating ``MaxwellUpdater``/``Simulation.step``.

    ``legacy=True`` reproduces core/solver.py:167-456 exactly (L0).
    ``legacy=False`` is the corrected stepper (L1) described in the package doc.
    """

    def __init__(self, grid: OracleGrid, dt: float, material_arrays: Optional[dict] = None,
                 legacy: bool = False, cpml_layers: int = 0, cpml_kwargs: Optional[dict] = None,
                 ade: Optional[Sequence[ADERegion]] = None, tfsf: Optional[TFSFPlane] = None):
        self.grid = grid
        self.dt = float(dt)
        self.legacy = legacy
        if grid.courant(dt) >= 1.0:  # core/solver.py:67-72
            raise ValueError("Time step violates Courant condition")
        nx, ny, nz = grid.dims
        ma = material_arrays or {}
        self.eps_rel = np.asarray(ma.get("eps_rel", np.ones((nx, ny, nz))), dtype=np.float64)
        self.mu_rel = np.asarray(ma.get("mu_rel", np.ones((nx, ny, nz))), dtype=np.float64)
        self.sigma_e = np.asarray(ma.get("sigma_e", np.zeros((nx, ny, nz))), dtype=np.float64)
        self.sigma_m = np.asarray(ma.get("sigma_m", np.zeros((nx, ny, nz))), dtype=np.float64)
        # core/solver.py:113-133
        eps = EPS0 * self.eps_rel
        s = self.sigma_e * self.dt / (2 * eps)
        self.Ca = (1 - s) / (1 + s)
        self.Cb = (self.dt / eps) / (1 + s)
        mu = MU0 * self.mu_rel
        sm = self.sigma_m * self.dt / (2 * mu)
        self.Da = (1 - sm) / (1 + sm)
        self.Db = (self.dt / mu) / (1 + sm)
        self.F = {c: np.zeros(grid.shape(c)) for c in COMPONENTS}
        # per-component interpolated coefficients
        if grid.is_2d:
            ip = lambda c, a: _interp2(c, a[:, :, 0])  # noqa: E731
        else:
            ip = _interp3
        self.ca = {c: ip(c, self.Ca) for c in ("Ex", "Ey", "Ez")}
        self.cb = {c: ip(c, self.Cb) for c in ("Ex", "Ey", "Ez")}
        self.da = {c: ip(c, self.Da) for c in ("Hx", "Hy", "Hz")}
        self.db = {c: ip(c, self.Db) for c in ("Hx", "Hy", "Hz")}
        # CPML per axis
        self.cpml_layers = cpml_layers
        self.pml = None
        if cpml_layers > 0:
            if legacy:
                raise ValueError("the reference stepper has no CPML")
            kw = dict(cpml_kwargs or {})
            dmax = max(grid.spacing)
            n_ax = [nx, ny] if grid.is_2d else [nx, ny, nz]
            self.pml = [cpml_profile(n, cpml_layers, dmax, self.dt, **kw) for n in n_ax]
        self.psi: dict = {}
        self.ade = list(ade or [])
        if self.ade and legacy:
            raise ValueError("the reference stepper has no ADE coupling")
        self._ade_state = []
        for reg in self.ade:
            ce, inv = ade_e_coefficients(reg.eps_inf, reg.poles, self.dt)
            st = {"ce": ce, "inv": inv, "comps": {}}
            for c in ("Ex", "Ey", "Ez"):
                sl = self._box_slices(c, reg.box)
                shp = self.F[c][sl].shape
                st["comps"][c] = {"sl": sl, "aux": [[np.zeros(shp), np.zeros(shp)] for _ in reg.poles]}
            self._ade_state.append(st)
        self.tfsf = tfsf
        if tfsf is not None:
            if legacy or grid.is_2d:
                raise ValueError("TFSF plane is implemented for the corrected 3D stepper")
            m = tfsf.m0 + int(math.ceil(0.5 * tfsf.max_steps * C0 * self.dt / grid.dz)) + 8
            self.aux_e = np.zeros(m)
            self.aux_h = np.zeros(m)
            self.aux_cb = self.dt / (EPS0 * tfsf.eps_b)
            self.aux_db = self.dt / MU0
        self.sources: list = []
        self.dfts: list = []
        self.time = 0.0
        self.step_count = 0

    # -- helpers -----------------------------------------------------------
    def _box_slices(self, comp, box):
        x0, x1, y0, y1, z0, z1 = box
        shp = self.F[comp].shape
        if self.grid.is_2d:
            return (slice(max(0, x0), min(x1, shp[0])), slice(max(0, y0), min(y1, shp[1])))
        return (slice(max(0, x0), min(x1, shp[0])), slice(max(0, y0), min(y1, shp[1])),
                slice(max(0, z0), min(z1, shp[2])))

    def _cp(self, name, d, axis, sl):
        """CPML-modified derivative kinv*d + psi, psi <- b psi + a d (Roden-Gedney)."""
        if self.pml is None:
            return d
        b, a, kap = self.pml[axis]
        shape = [1] * d.ndim
        bb, aa, kk = b[sl], a[sl], kap[sl]
        shape[axis] = bb.size
        bb, aa, kk = bb.reshape(shape), aa.reshape(shape), kk.reshape(shape)
        psi = self.psi.get(name)
        if psi is None:
            psi = np.zeros(d.shape)
            self.psi[name] = psi
        psi *= bb
        psi += aa * d
        return d / kk + psi

    # -- sources / monitors (Simulation.step, core/simulation.py:147-164) ----
    def add_source(self, comp, index, waveform, weight=1.0):
        self.sources.append(_Source(comp, index, weight, waveform))

    def add_dft(self, comp, index, freqs):
        shp = self.F[comp][index].shape
        d = _DFT(comp, index, np.asarray(freqs, dtype=np.float64))
        d.data = np.zeros((len(d.freqs),) + shp, dtype=np.complex128)
        self.dfts.append(d)
        return len(self.dfts) - 1

    # -- stepping ------------------------------------------------------------
    def step(self):
        g = self.grid
        if self.legacy:
            (self._h2_legacy if g.is_2d else self._h3_legacy)()
            (self._e2 if g.is_2d else self._e3)()
        else:
            (self._h2 if g.is_2d else self._h3)()
            if self.tfsf is not None:
                self._tfsf_h()
            (self._e2 if g.is_2d else self._e3)()
            if self.tfsf is not None:
                self._tfsf_e()
        # core/simulation.py:155-164: time advances, then sources, then monitors
        self.step_count += 1
        self.time += self.dt
        t = self.time
        if self.tfsf is not None:
            self.aux_e[0] = self.tfsf.waveform(t)
        for s in self.sources:
            self.F[s.comp][s.index] += s.weight * s.waveform(t)
        for d in self.dfts:
            fd = self.F[d.comp][d.index]
            for fi, f in enumerate(d.freqs):
                omega = 2 * np.pi * f  # monitors/field.py:140-143
                d.data[fi] += fd * np.exp(-1j * omega * t) * self.dt

    def run(self, n):
        for _ in range(n):
            self.step()

    # -- L1 (corrected) 3D --------------------------------------------------
    def _h3(self):
        F = self.F
        dx, dy, dz = self.grid.spacing
        Ex, Ey, Ez, Hx, Hy, Hz = (F[c] for c in COMPONENTS)
        inner = slice(1, -1)
        # Hx(:, 1:-1, 1:-1)
        r = (slice(None), inner, inner)
        cy = self._cp("Hxy", (Ez[:, 1:, 1:-1] - Ez[:, :-1, 1:-1]) / dy, 1, inner)
        cz = self._cp("Hxz", (Ey[:, 1:-1, 1:] - Ey[:, 1:-1, :-1]) / dz, 2, inner)
        Hx[r] = self.da["Hx"][r] * Hx[r] - self.db["Hx"][r] * (cy - cz)
        # Hy(1:-1, :, 1:-1)
        r = (inner, slice(None), inner)
        cz = self._cp("Hyz", (Ex[1:-1, :, 1:] - Ex[1:-1, :, :-1]) / dz, 2, inner)
        cx = self._cp("Hyx", (Ez[1:, :, 1:-1] - Ez[:-1, :, 1:-1]) / dx, 0, inner)
        Hy[r] = self.da["Hy"][r] * Hy[r] - self.db["Hy"][r] * (cz - cx)
        # Hz(1:-1, 1:-1, :)
        r = (inner, inner, slice(None))
        cx = self._cp("Hzx", (Ey[1:, 1:-1, :] - Ey[:-1, 1:-1, :]) / dx, 0, inner)
        cy = self._cp("Hzy", (Ex[1:-1, 1:, :] - Ex[1:-1, :-1, :]) / dy, 1, inner)
        Hz[r] = self.da["Hz"][r] * Hz[r] - self.db["Hz"][r] * (cx - cy)

    def _e3(self):
        F = self.F
        dx, dy, dz = self.grid.spacing
        nx, ny, nz = self.grid.dims
        Ex, Ey, Ez, Hx, Hy, Hz = (F[c] for c in COMPONENTS)
        sx, sy, sz = slice(0, nx - 1), slice(0, ny - 1), slice(0, nz - 1)
        curl = {}
        curl["Ex"] = (self._cp("Exy", (Hz[:, 1:, :] - Hz[:, :-1, :]) / dy, 1, sy)
                      - self._cp("Exz", (Hy[:, :, 1:] - Hy[:, :, :-1]) / dz, 2, sz))
        curl["Ey"] = (self._cp("Eyz", (Hx[:, :, 1:] - Hx[:, :, :-1]) / dz, 2, sz)
                      - self._cp("Eyx", (Hz[1:, :, :] - Hz[:-1, :, :]) / dx, 0, sx))
        curl["Ez"] = (self._cp("Ezx", (Hy[1:, :, :] - Hy[:-1, :, :]) / dx, 0, sx)
                      - self._cp("Ezy", (Hx[:, 1:, :] - Hx[:, :-1, :]) / dy, 1, sy))
        self._apply_e(curl)

    def _apply_e(self, curl):
        F = self.F
        old = {}
        for st in self._ade_state:
            for c, cs in st["comps"].items():
                old[(id(st), c)] = F[c][cs["sl"]].copy()
        for c in ("Ex", "Ey", "Ez"):
            if c in curl:
                F[c][...] = self.ca[c] * F[c] + self.cb[c] * curl[c]
        # ADE regions override the plain update (see ade_e_coefficients)
        for reg, st in zip(self.ade, self._ade_state):
            for c, cs in st["comps"].items():
                if c not in curl:
                    continue
                sl = cs["sl"]
                e_old = old[(id(st), c)]
                s_term = (self.dt / EPS0) * curl[c][sl]
                acc = st["ce"] * e_old + st["inv"] * s_term
                for p, (a0, a1) in zip(reg.poles, cs["aux"]):
                    if p["kind"] == "lorentz":
                        acc -= st["inv"] * ((p["C2"] - 1.0) * a0 + p["C3"] * a1)
                    elif p["kind"] == "drude":
                        acc -= st["inv"] * (0.5 * self.dt * (1.0 + p["C1"]) * a0)
                    else:  # debye
                        acc -= st["inv"] * ((p["C1"] - 1.0) * a0)
                e_new = acc
                for p, aux in zip(reg.poles, cs["aux"]):
                    a0, a1 = aux
                    if p["kind"] == "lorentz":
                        pn = p["C0"] * e_new + p["C1"] * e_old + p["C2"] * a0 + p["C3"] * a1
                        aux[1] = a0
                        aux[0] = pn
                    elif p["kind"] == "drude":
                        aux[0] = p["C1"] * a0 + p["C0"] * 0.5 * (e_new + e_old)
                    else:
                        aux[0] = p["C1"] * a0 + p["C0"] * 0.5 * (e_new + e_old)
                F[c][sl] = e_new

    # -- L1 (corrected) 2D --------------------------------------------------
    def _h2(self):
        F = self.F
        dx, dy, _ = self.grid.spacing
        Ex, Ey, Ez, Hx, Hy, Hz = (F[c] for c in COMPONENTS)
        inner = slice(1, -1)
        r = (slice(None), inner)
        Hx[r] = self.da["Hx"][r] * Hx[r] - self.db["Hx"][r] * self._cp("Hxy", (Ez[:, 1:] - Ez[:, :-1]) / dy, 1, inner)
        r = (inner, slice(None))
        Hy[r] = self.da["Hy"][r] * Hy[r] + self.db["Hy"][r] * self._cp("Hyx", (Ez[1:, :] - Ez[:-1, :]) / dx, 0, inner)
        r = (inner, inner)
        cx = self._cp("Hzx", (Ey[1:, 1:-1] - Ey[:-1, 1:-1]) / dx, 0, inner)
        cy = self._cp("Hzy", (Ex[1:-1, 1:] - Ex[1:-1, :-1]) / dy, 1, inner)
        Hz[r] = self.da["Hz"][r] * Hz[r] - self.db["Hz"][r] * (cx - cy)

    def _e2(self):
        F = self.F
        dx, dy, _ = self.grid.spacing
        nx, ny, _ = self.grid.dims
        Ex, Ey, Ez, Hx, Hy, Hz = (F[c] for c in COMPONENTS)
        sx, sy = slice(0, nx - 1), slice(0, ny - 1)
        if self.legacy:
            # core/solver.py:399-456 (no CPML in the reference)
            curl = {
                "Ez": (Hy[1:, :] - Hy[:-1, :]) / dx - (Hx[:, 1:] - Hx[:, :-1]) / dy,
                "Ex": (Hz[:, 1:] - Hz[:, :-1]) / dy,
                "Ey": -(Hz[1:, :] - Hz[:-1, :]) / dx,
            }
        else:
            curl = {
                "Ez": (self._cp("Ezx", (Hy[1:, :] - Hy[:-1, :]) / dx, 0, sx)
                       - self._cp("Ezy", (Hx[:, 1:] - Hx[:, :-1]) / dy, 1, sy)),
                "Ex": self._cp("Exy", (Hz[:, 1:] - Hz[:, :-1]) / dy, 1, sy),
                "Ey": -self._cp("Eyx", (Hz[1:, :] - Hz[:-1, :]) / dx, 0, sx),
            }
        self._apply_e(curl)

    # -- L0 (reference-exact) ----------------------------------------------
    def _h3_legacy(self):
        """core/solver.py:167-253 verbatim semantics (forward diffs into [:-2] slices)."""
        F = self.F
        dx, dy, dz = self.grid.spacing
        Ex, Ey, Ez, Hx, Hy, Hz = (F[c] for c in COMPONENTS)
        nx, ny, nz = self.grid.dims
        cy = (Ez[:, 1:, :] - Ez[:, :-1, :]) / dy
        cz = (Ey[:, :, 1:] - Ey[:, :, :-1]) / dz
        a, b = ny - 2, nz - 2
        Hx[:, :a, :b] = self.da["Hx"][:, :a, :b] * Hx[:, :a, :b] - self.db["Hx"][:, :a, :b] * (cy[:, :a, :b] - cz[:, :a, :b])
        cz = (Ex[:, :, 1:] - Ex[:, :, :-1]) / dz
        cx = (Ez[1:, :, :] - Ez[:-1, :, :]) / dx
        a, b = nx - 2, nz - 2
        Hy[:a, :, :b] = self.da["Hy"][:a, :, :b] * Hy[:a, :, :b] - self.db["Hy"][:a, :, :b] * (cz[:a, :, :b] - cx[:a, :, :b])
        cx = (Ey[1:, :, :] - Ey[:-1, :, :]) / dx
        cy = (Ex[:, 1:, :] - Ex[:, :-1, :]) / dy
        a, b = nx - 2, ny - 2
        Hz[:a, :b, :] = self.da["Hz"][:a, :b, :] * Hz[:a, :b, :] - self.db["Hz"][:a, :b, :] * (cx[:a, :b, :] - cy[:a, :b, :])

    def _h2_legacy(self):
        """core/solver.py:311-397 verbatim semantics (sign flips, family skip)."""
        F = self.F
        dx, dy, _ = self.grid.spacing
        Ex, Ey, Ez, Hx, Hy, Hz = (F[c] for c in COMPONENTS)
        nx, ny, _ = self.grid.dims
        if np.max(np.abs(Ez)) > 0:
            cy = (Ez[:, 1:] - Ez[:, :-1]) / dy
            a = ny - 2
            Hx[:, :a] = self.da["Hx"][:, :a] * Hx[:, :a] + self.db["Hx"][:, :a] * cy[:, :a]
            cx = (Ez[1:, :] - Ez[:-1, :]) / dx
            a = nx - 2
            Hy[:a, :] = self.da["Hy"][:a, :] * Hy[:a, :] - self.db["Hy"][:a, :] * cx[:a, :]
        if np.max(np.abs(Ex)) > 0 or np.max(np.abs(Ey)) > 0:
            cx = np.zeros_like(Hz)
            if Ey.shape[0] > 1:
                a = min(Ey.shape[0] - 1, Hz.shape[0] - 1)
                cx[:a, :] = (Ey[1:a + 1, :] - Ey[:a, :]) / dx
            cy = np.zeros_like(Hz)
            if Ex.shape[1] > 1:
                a = min(Ex.shape[1] - 1, Hz.shape[1] - 1)
                cy[:, :a] = (Ex[:, 1:a + 1] - Ex[:, :a]) / dy
            Hz[:, :] = self.da["Hz"] * Hz - self.db["Hz"] * (cx - cy)

    # -- TFSF plane ---------------------------------------------------------
    def _tfsf_sign_h(self):
        t = self.tfsf
        s = 1.0 if t.direction > 0 else -1.0
        return s if t.polarization == "x" else -s

    def _tfsf_h(self):
        """Correct H next to the plane with the incident E at time n, then advance
        the auxiliary H to n+1/2."""
        t = self.tfsf
        dz = self.grid.dz
        hc = "Hy" if t.polarization == "x" else "Hx"
        kh = t.k0 if t.direction > 0 else t.k0 + 1
        H = self.F[hc]
        db = self.db[hc][:, :, kh]
        inner_i = slice(1, -1) if hc == "Hy" else slice(None)
        inner_j = slice(None) if hc == "Hy" else slice(1, -1)
        H[inner_i, inner_j, kh] += self._tfsf_sign_h() * db[inner_i, inner_j] * self.aux_e[t.m0] / dz
        # auxiliary 1D grid: h -= Db (e[m] - e[m-1]) / dz
        self.aux_h[1:-1] -= self.aux_db * (self.aux_e[1:-1] - self.aux_e[:-2]) / dz

    def _tfsf_e(self):
        t = self.tfsf
        dz = self.grid.dz
        ec = "Ex" if t.polarization == "x" else "Ey"
        E = self.F[ec]
        E[:, :, t.k0] += self.cb[ec][:, :, t.k0] * self.aux_h[t.m0] / dz
        # auxiliary 1D grid: e -= Cb (h[m+1] - h[m]) / dz
        self.aux_e[:-1] -= self.aux_cb * (self.aux_h[1:] - self.aux_h[:-1]) / dz


def field_energy(F, grid, eps_e=None):
    """Discrete field energy 0.5 (eps0 |E|^2 + mu0 |H|^2) dV (core/fields.py:237-285)."""
    dV = grid.dx * grid.dy * (grid.dz if not grid.is_2d else 1.0)
    e = sum(np.sum(F[c] ** 2) for c in ("Ex", "Ey", "Ez"))
    h = sum(np.sum(F[c] ** 2) for c in ("Hx", "Hy", "Hz"))
    return 0.5 * EPS0 * e * dV + 0.5 * MU0 * h * dV
