"""Batched 2D directional-coupler sweep on the device (pc_batch_* C ABI).

The reference sweeps a design space one simulation at a time
(``ParameterSweep``, optimization/sweep.py:41-195: a Python loop, or a process
pool, around ``Simulation.run``) and extracts port amplitudes with a mode
overlap (utils/mode_matching.py:41-131).  Here a whole family of 2D TE designs
of uneven size runs as one batch: every design's Ez/Hx/Hy live in shared device
buffers, one persistent kernel per pass advances all of them, and the time loop
is replayed from a CUDA graph (csrc/batch.cu).

Workload (directional couplers, 20 nm cells, 20-cell CPML, Courant 0.5):

* design ``seed``: Nx ~ U{400..1200}, Ny ~ U{200..800}, strip width ~ U[0.4, 0.6] um,
  gap ~ U[0.1, 0.4] um, coupling length ~ U[2, 10] um; Si (12.11) in SiO2 (2.085).
* guide A is straight; guide B runs beside it over the coupling length and
  leaves through straight leads offset 0.8 um further away, joined to the
  coupling section by short lateral jogs (straight port leads instead of
  S-bends).  The coupling section starts a fixed distance after the input
  ports and the output ports sit a fixed distance after it, so the domain is
  lengthened when Nx is too short for the drawn length (``CouplerLayout.nx``).
* cells on a strip edge take the strip's area fraction (fill-fraction
  permittivity), so the S-parameters vary continuously with width, gap and
  length; the reference's point sampling (geometry/shapes.py:71-132) would make
  them piecewise constant in the 20 nm grid.
* a soft Ez line source with the TE0 profile of guide A (Gaussian pulse 193 THz,
  10 fs) at x = CPML + 10; port DFT lines of Ez at 64 frequencies for
  wavelengths 1.5-1.6 um: port 1 (A, input side), 2 (A, output), 3 (B, output),
  4 (B, input side).
* every design has a normalisation instance: guide A alone in a short domain
  with the same source and port 1.
* port amplitude a_k(f) = sum_y Ez_k(y, f) m_k(y) / sum_y m_k(y)^2 with the
  port's TE0 profile m_k (the Ez part of the overlap of mode_matching.py:41-131);
  S11 = (a_1 - a_1^norm) / a_1^norm, S_k1 = a_k / a_1^norm (k = 2, 3, 4).

The TE0 profiles come from a finite-difference eigenproblem across the strip
(as modes/solver.py:135-226 does in 2D), solved with the Yee scheme's own
discrete operators in time and x, so that the propagation constant ``beta`` is
the one the FDTD grid actually carries; ``deembed`` uses it to move the output
reference planes, which removes the fast phase exp(-i beta L) from the spectra.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from . import _lib
from .pml import PMLParams, cpml_axis_coefficients
from .sources import GaussianPulse

C0 = 299792458.0
EPS0 = 8.854187817e-12
MU0 = 4 * np.pi * 1e-7
EPS_SI = 12.11
EPS_SIO2 = 2.085

DX = 20e-9
CPML = 20
COURANT = 0.5
STEPS = 4000
NFREQ = 64
F0 = 193e12
PULSE_WIDTH = 10e-15

SRC_OFF = 10  # source column: CPML + 10
PORT_OFF = 15  # input ports 15 cells after the source
GAP_IN = 20  # cells from the input ports to the coupling section, and from it to the output ports
TAIL = 15  # cells from the output ports to the CPML
LEAD_OFFSET = 0.8e-6  # guide B's leads sit this much further from guide A than its coupling section
WINDOW_MARGIN = 0.4e-6  # port window: strip +- this margin
NORM_TAIL = 40  # normalisation domain: cells from port 1 to the CPML


def sweep_dt(dx: float = DX) -> float:
    """Courant 0.5 on a square 2D grid (core/grid.py:258-326)."""
    return COURANT / (C0 * math.sqrt(2.0 / dx**2))


def sweep_freqs(n: int = NFREQ) -> np.ndarray:
    return C0 / np.linspace(1.5e-6, 1.6e-6, n)


# ---------------------------------------------------------------------------
# geometry
# ---------------------------------------------------------------------------
@dataclass
class CouplerDesign:
    seed: int
    nx: int
    ny: int
    width: float
    gap: float
    length: float

    def params(self) -> np.ndarray:
        """(width, gap, length) normalised to [0, 1] over their sampling ranges."""
        return np.array([(self.width - 0.4e-6) / 0.2e-6, (self.gap - 0.1e-6) / 0.3e-6,
                         (self.length - 2e-6) / 8e-6])


def coupler_design(seed: int) -> CouplerDesign:
    rng = np.random.default_rng(seed)
    nx = int(rng.integers(400, 1201))
    ny = int(rng.integers(200, 801))
    width = float(rng.uniform(0.4e-6, 0.6e-6))
    gap = float(rng.uniform(0.1e-6, 0.4e-6))
    length = float(rng.uniform(2e-6, 10e-6))
    return CouplerDesign(seed, nx, ny, width, gap, length)


def design_from_params(p, nx: int = 400, ny: int = 200, seed: int = -1) -> CouplerDesign:
    p = np.asarray(p, dtype=np.float64)
    return CouplerDesign(seed, nx, ny, 0.4e-6 + 0.2e-6 * p[0], 0.1e-6 + 0.3e-6 * p[1], 2e-6 + 8e-6 * p[2])


def _overlap(n: int, d: float, lo: float, hi: float) -> np.ndarray:
    """Length of [lo, hi] inside each cell [i d, (i+1) d], in cells."""
    edges = np.arange(n + 1) * d
    return np.clip(np.minimum(edges[1:], hi) - np.maximum(edges[:-1], lo), 0.0, None) / d


def fill_eps(nx: int, ny: int, rects, d: float, eps_core: float = EPS_SI, eps_clad: float = EPS_SIO2):
    """Cell-centred permittivity of non-overlapping rectangles (x0, x1, y0, y1) in metres,
    each cell weighted by the area fraction it shares with the strips.  The area
    fractions are accumulated over the band of y cells the strips touch only (the
    cladding elsewhere gets the same value, eps_clad + (eps_core - eps_clad) * 0)."""
    blocks = []
    for x0, x1, y0, y1 in rects:
        ox, oy = _overlap(nx, d, x0, x1), _overlap(ny, d, y0, y1)
        ix, iy = np.nonzero(ox)[0], np.nonzero(oy)[0]
        if ix.size and iy.size:  # the strip's own block of cells only
            blocks.append((ix[0], ix[-1] + 1, iy[0], iy[-1] + 1, ox, oy))
    eps = np.full((nx, ny), float(eps_clad))
    if not blocks:
        return eps
    b0, b1 = min(b[2] for b in blocks), max(b[3] for b in blocks)
    fill = np.zeros((nx, b1 - b0))
    for i0, i1, j0, j1, ox, oy in blocks:
        fill[i0:i1, j0 - b0:j1 - b0] += np.outer(ox[i0:i1], oy[j0:j1])
    np.clip(fill, 0.0, 1.0, out=fill)
    fill *= eps_core - eps_clad
    fill += eps_clad
    eps[:, b0:b1] = fill
    return eps


@dataclass
class Port:
    x: int  # Ez index along x
    y0: int  # first Ez index along y
    n: int
    profile: np.ndarray = field(repr=False)  # TE0 profile on the window (max 1)


@dataclass
class CouplerLayout:
    design: CouplerDesign
    nx: int
    ny: int
    eps: np.ndarray  # (nx, ny) cell-centred
    src: Port  # line source (window and weights)
    ports: List[Port]  # 1, 2, 3, 4
    norm_nx: int
    norm_eps: np.ndarray
    y_a: float
    y_lead: float
    xc0: float  # coupling section start (m)
    length: float  # coupling section length (m)

    @property
    def path(self) -> float:
        """Distance from the input to the output ports (m)."""
        return (self.ports[1].x - self.ports[0].x) * DX


def _window(ny: int, yc: float, w: float, d: float, cpml: int):
    jpos = (np.arange(ny - 1) + 1) * d  # Ez sits at y = (j + 1) d
    sel = np.nonzero(np.abs(jpos - yc) <= w / 2 + WINDOW_MARGIN)[0]
    sel = sel[(sel >= cpml) & (sel < ny - 1 - cpml)]
    return int(sel[0]), int(sel.size)


def _ez_eps_line(eps: np.ndarray, x: int, y0: int, n: int) -> np.ndarray:
    """Permittivity at Ez points of column x (the 4-point mean the coefficients use)."""
    e = eps
    return 0.25 * (e[x, y0:y0 + n] + e[x + 1, y0:y0 + n] + e[x, y0 + 1:y0 + n + 1] + e[x + 1, y0 + 1:y0 + n + 1])


def te0_mode(eps_line: np.ndarray, d: float, freq: float, dt: float):
    """TE0 (Ez) profile and propagation constant of a 2D slab on the Yee grid.

    Discrete Helmholtz operator across the strip (second difference, zero outside
    the window) with the scheme's temporal and x operators:
        (2/(c dt))^2 sin^2(w dt/2) eps m + D_yy m = mu m,
        (2/dx)^2 sin^2(beta dx/2) = mu,
    largest mu = TE0.  Returns (profile with max 1, beta)."""
    from scipy.linalg import eigh_tridiagonal

    k2 = (2.0 / (C0 * dt)) ** 2 * math.sin(math.pi * freq * dt) ** 2
    n = eps_line.size
    diag = k2 * eps_line - 2.0 / d**2
    off = np.full(n - 1, 1.0 / d**2)
    mu, vec = eigh_tridiagonal(diag, off, select="i", select_range=(n - 1, n - 1))
    v = vec[:, 0]
    v = v / v[np.argmax(np.abs(v))]
    s = min(1.0, d * math.sqrt(max(mu[0], 0.0)) / 2.0)
    beta = 2.0 / d * math.asin(s)
    return v, beta


def te0_beta(eps_line: np.ndarray, d: float, freqs: np.ndarray, dt: float) -> np.ndarray:
    from scipy.linalg import eigvalsh_tridiagonal

    n = eps_line.size
    off = np.full(n - 1, 1.0 / d**2)
    out = np.empty(len(freqs))
    for q, f in enumerate(freqs):
        k2 = (2.0 / (C0 * dt)) ** 2 * math.sin(math.pi * f * dt) ** 2
        mu = eigvalsh_tridiagonal(k2 * eps_line - 2.0 / d**2, off, select="i", select_range=(n - 1, n - 1))[0]
        out[q] = 2.0 / d * math.asin(min(1.0, d * math.sqrt(max(mu, 0.0)) / 2.0))
    return out


def coupler_layout(design: CouplerDesign, d: float = DX, cpml: int = CPML) -> CouplerLayout:
    w, g, L = design.width, design.gap, design.length
    dt = sweep_dt(d)
    src_x = cpml + SRC_OFF
    p1 = src_x + PORT_OFF
    xc0 = (p1 + 1 + GAP_IN) * d
    xe = xc0 + L
    p2 = int(math.ceil(xe / d + GAP_IN - 1))
    nx = max(design.nx, p2 + TAIL + cpml + 2)
    ny = design.ny
    height = 2 * w + g + LEAD_OFFSET
    y_top = ny * d / 2 + height / 2
    y_a = y_top - w / 2
    y_b = y_a - (w + g)
    y_l = y_b - LEAD_OFFSET
    X = nx * d
    rects = [
        (0.0, X, y_a - w / 2, y_a + w / 2),  # guide A
        (0.0, xc0 - w, y_l - w / 2, y_l + w / 2),  # B input lead
        (xc0 - w, xc0, y_l - w / 2, y_b + w / 2),  # jog
        (xc0, xe, y_b - w / 2, y_b + w / 2),  # coupling section
        (xe, xe + w, y_l - w / 2, y_b + w / 2),  # jog
        (xe + w, X, y_l - w / 2, y_l + w / 2),  # B output lead
    ]
    eps = fill_eps(nx, ny, rects, d)
    ports = []
    for x, yc in ((p1, y_a), (p2, y_a), (p2, y_l), (p1, y_l)):
        y0, n = _window(ny, yc, w, d, cpml)
        prof, _ = te0_mode(_ez_eps_line(eps, x, y0, n), d, F0, dt)
        ports.append(Port(x, y0, n, prof))
    y0, n = _window(ny, y_a, w, d, cpml)
    sprof, _ = te0_mode(_ez_eps_line(eps, src_x, y0, n), d, F0, dt)
    src = Port(src_x, y0, n, sprof)
    norm_nx = p1 + NORM_TAIL + cpml + 2
    norm_eps = fill_eps(norm_nx, ny, [(0.0, norm_nx * d, y_a - w / 2, y_a + w / 2)], d)
    return CouplerLayout(design, nx, ny, eps, src, ports, norm_nx, norm_eps, y_a, y_l, xc0, L)


def amplitudes(nsteps: int, dt: float) -> np.ndarray:
    """a(t_{n+1}) of the sweep's Gaussian pulse for steps 0..nsteps-1."""
    return GaussianPulse(F0, PULSE_WIDTH).evaluate((np.arange(nsteps) + 1) * dt)


# ---------------------------------------------------------------------------
# S-parameters
# ---------------------------------------------------------------------------
def port_amplitude(spec: np.ndarray, profile: np.ndarray) -> np.ndarray:
    """spec (nf, n) complex DFT of Ez on a port line -> (nf,) modal amplitude."""
    return spec @ profile / float(profile @ profile)


def s_parameters(coupler_spec: Sequence[np.ndarray], norm_spec: np.ndarray, layout: CouplerLayout) -> np.ndarray:
    """(4, nf) complex S11, S21, S31, S41."""
    a = [port_amplitude(s, p.profile) for s, p in zip(coupler_spec, layout.ports)]
    inc = port_amplitude(norm_spec, layout.ports[0].profile)
    return np.stack([(a[0] - inc) / inc, a[1] / inc, a[2] / inc, a[3] / inc])


def deembed(S: np.ndarray, layout: CouplerLayout, freqs: np.ndarray, dt: Optional[float] = None,
            inverse: bool = False) -> np.ndarray:
    """Move the reference planes by the TE0 propagation phase: S21, S31 by the
    input-to-output port distance, S11, S41 by twice the distance from the input
    ports to the coupling section.  ``inverse`` puts the phase back."""
    dt = dt or sweep_dt()
    p = layout.ports[0]
    beta = te0_beta(_ez_eps_line(layout.norm_eps, p.x, p.y0, p.n), DX, freqs, dt)
    return apply_phase(S, beta, layout, inverse)


def apply_phase(S, beta, layout: CouplerLayout, inverse: bool = False):
    back = 2.0 * (layout.xc0 - (layout.ports[0].x + 1) * DX)
    dist = np.array([back, layout.path, layout.path, back])
    ph = np.exp((-1j if inverse else 1j) * beta[None, :] * dist[:, None])
    return S * ph


# ---------------------------------------------------------------------------
# batched FDTD through the C ABI
# ---------------------------------------------------------------------------
@dataclass
class Instance:
    eps: np.ndarray  # (nx, ny)
    src: Port
    ports: List[Port]


def instances_for(layouts: Sequence[CouplerLayout]) -> List[Instance]:
    """Coupler then normalisation instance of every layout."""
    out = []
    for L in layouts:
        out.append(Instance(L.eps, L.src, L.ports))
        out.append(Instance(L.norm_eps, L.src, [L.ports[0]]))
    return out


class BatchedFDTD2D:
    """Many 2D TE simulations advanced together on one GPU.

    Buffers (field sets, Cb, CPML auxiliaries, DFT accumulators) are torch
    tensors owned here; the native batch holds raw pointers to them."""

    def __init__(self, instances: Sequence[Instance], freqs, dx: float = DX, dt: Optional[float] = None,
                 cpml: int = CPML, device=None, stream=None, autotune: bool = True, graph_steps: int = 80,
                 variant: Optional[int] = None, field_sets=None, dft_t0: Optional[float] = None):
        """``field_sets`` (one instance only): two float32 tensors whose storage
        from their first element holds that instance's Ez, Hx, Hy ([3][nx][pitch],
        pitch = ny rounded up to 32) -- the batch steps them in place instead of
        buffers of its own.  ``dft_t0``: time of the first DFT sample (default dt)."""
        import torch

        self.torch = torch
        self.lib = _lib.load()
        self.device = torch.device(device or "cuda")
        if self.device.type != "cuda":
            raise RuntimeError("the batched sweep runs on a CUDA device only")
        self.stream = stream or torch.cuda.current_stream(self.device)
        self.dx = dx
        self.dt = dt or sweep_dt(dx)
        self.cpml = cpml
        self.freqs = np.asarray(freqs, dtype=np.float64)
        self.instances = list(instances)
        n = len(self.instances)
        arr = (_lib.BatchInstance * n)()
        for q, I in enumerate(self.instances):
            a = arr[q]
            a.nx, a.ny = I.eps.shape
            a.src_x, a.src_y0, a.src_n = I.src.x, I.src.y0, I.src.n
            a.nport = len(I.ports)
            for k, p in enumerate(I.ports):
                a.port_x[k], a.port_y0[k], a.port_n[k] = p.x, p.y0, p.n
        self.lay = _lib.BatchLayout()
        h = C.c_void_p()
        _lib.check(self.lib.pc_batch_create(n, arr, cpml, dx, dx, self.dt, self.dt / MU0, C.byref(h),
                                            C.byref(self.lay)), "pc_batch_create")
        self.h = h
        lay = self.lay
        dev, f32 = self.device, torch.float32
        with torch.cuda.device(dev):
            if field_sets is not None:
                if n != 1 or len(field_sets) != 2 or any(t.dtype != f32 or not t.is_contiguous() or
                                                          t.numel() < lay.field_elems for t in field_sets):
                    self.lib.pc_batch_destroy(h)
                    self.h = None
                    raise ValueError("external field sets: one instance, two contiguous float32 tensors")
                self.sets = list(field_sets)
            else:
                self.sets = [torch.zeros(lay.field_elems, dtype=f32, device=dev) for _ in range(2)]
            self.cb = torch.zeros(lay.coef_elems, dtype=f32, device=dev)
            self.psi = [torch.zeros(lay.psi_elems, dtype=f32, device=dev) for _ in range(2)]
            self.acc = torch.zeros((len(self.freqs), lay.dft_points, 4), dtype=f32, device=dev)
        sp = self.stream.cuda_stream
        _lib.check(self.lib.pc_batch_bind(h, self.sets[0].data_ptr(), self.sets[1].data_ptr(), self.cb.data_ptr(),
                                          self.psi[0].data_ptr(), self.psi[1].data_ptr()), "pc_batch_bind")
        self.offsets = []
        for q in range(n):
            o = (C.c_int64 * 5)()
            _lib.check(self.lib.pc_batch_instance_offsets(h, q, o), "pc_batch_instance_offsets")
            self.offsets.append(tuple(int(v) for v in o))
        # every instance's permittivity in one pinned upload, then the builds back to back
        sizes = [I.eps.size for I in self.instances]
        starts = np.concatenate([[0], np.cumsum(sizes)])
        host = torch.empty(int(starts[-1]), dtype=torch.float64, pin_memory=True)
        hv = host.numpy()
        for q, I in enumerate(self.instances):
            hv[starts[q]:starts[q + 1]] = I.eps.ravel()
        with torch.cuda.stream(self.stream):
            eps_all = host.to(dev, non_blocking=True)
        for q in range(n):
            ptr = eps_all.data_ptr() + int(starts[q]) * 8
            _lib.check(self.lib.pc_batch_build_coefficients(h, q, ptr, EPS0, sp), "pc_batch_build_coefficients")
        self.stream.synchronize()
        del eps_all, host
        if cpml > 0:
            b, a, k = cpml_axis_coefficients(2 * cpml + 2, PMLParams(cpml), max(dx, dx), self.dt)
            sl = np.r_[0:cpml, cpml + 2:2 * cpml + 2]  # lower slab, then upper slab, by slab index
            D = C.POINTER(C.c_double)
            bs, as_, ks = (np.ascontiguousarray(v[sl]) for v in (b, a, k))
            _lib.check(self.lib.pc_batch_set_cpml(h, bs.ctypes.data_as(D), as_.ctypes.data_as(D),
                                                  ks.ctypes.data_as(D)), "pc_batch_set_cpml")
        self._w = np.ascontiguousarray(np.concatenate([I.src.profile for I in self.instances]), dtype=np.float64)
        om = np.ascontiguousarray(2 * np.pi * self.freqs)
        if lay.dft_points > 0:
            _lib.check(self.lib.pc_batch_set_dft(h, om.ctypes.data_as(C.POINTER(C.c_double)), int(om.size),
                                                 self.dt if dft_t0 is None else float(dft_t0), self.acc.data_ptr()),
                       "pc_batch_set_dft")
        self.set_amplitudes(np.zeros(0))
        self.tuning_ms = None
        if variant is not None:
            self.set_tuning(variant, graph_steps)
        elif autotune:
            self.autotune(graph_steps=graph_steps)
        else:
            self.set_tuning(1, graph_steps)

    # -- setup ------------------------------------------------------------------
    def set_amplitudes(self, amps: np.ndarray):
        a = np.ascontiguousarray(amps, dtype=np.float64)
        self._amps = a
        D = C.POINTER(C.c_double)
        _lib.check(self.lib.pc_batch_set_sources(self.h, self._w.ctypes.data_as(D), a.ctypes.data_as(D), int(a.size)),
                   "pc_batch_set_sources")

    @staticmethod
    def variants():
        lib = _lib.load()
        out = []
        for v in range(lib.pc_batch_num_variants()):
            o = (C.c_int32 * 3)()
            _lib.check(lib.pc_batch_variant_info(v, o), "pc_batch_variant_info")
            out.append(tuple(int(x) for x in o))
        return out

    def set_tuning(self, variant: int, graph_steps: int = 80):
        _lib.check(self.lib.pc_batch_set_tuning(self.h, int(variant), int(graph_steps)), "pc_batch_set_tuning")

    def tuning(self):
        v, g = C.c_int32(), C.c_int32()
        _lib.check(self.lib.pc_batch_get_tuning(self.h, C.byref(v), C.byref(g)), "pc_batch_get_tuning")
        return int(v.value), int(g.value)

    def autotune(self, passes: int = 4, graph_steps: int = 80):
        """Time dry passes of every kernel variant (tile shape, steps per pass) on
        this batch and keep the fastest; graph_steps is rounded to a multiple of
        16 steps holding an even number of passes."""
        nv = self.lib.pc_batch_num_variants()
        ms = (C.c_float * nv)()
        _lib.check(self.lib.pc_batch_autotune(self.h, int(passes), ms, self.stream.cuda_stream), "pc_batch_autotune")
        self.tuning_ms = [float(x) for x in ms]
        v, _ = self.tuning()
        k = self.variants()[v][2]
        unit = int(np.lcm(16, 2 * k))
        g = max(unit, (graph_steps // unit) * unit) if graph_steps > 0 else 0
        self.set_tuning(v, g)
        return v

    # -- stepping -----------------------------------------------------------------
    def step(self, nsteps: int):
        _lib.check(self.lib.pc_batch_step(self.h, int(nsteps), self.stream.cuda_stream), "pc_batch_step")

    def run(self, nsteps: int = STEPS):
        """Drive every instance with the sweep pulse for nsteps (from the current step)."""
        done = self.steps_done
        self.set_amplitudes(amplitudes(done + nsteps, self.dt))
        self.step(nsteps)

    @property
    def steps_done(self) -> int:
        return int(self.lib.pc_batch_steps_done(self.h))

    @property
    def launches(self) -> int:
        return int(self.lib.pc_batch_launch_count(self.h))

    @property
    def cur(self) -> int:
        return int(self.lib.pc_batch_current_set(self.h))

    def status(self) -> int:
        """The batch's PC_STATUS_* word."""
        v = C.c_uint32(0)
        _lib.check(self.lib.pc_batch_status(self.h, C.byref(v), self.stream.cuda_stream), "pc_batch_status")
        return int(v.value)

    def instance_status(self) -> np.ndarray:
        """Per-instance PC_STATUS_* words since the last read (then cleared):
        PC_STATUS_NONFINITE marks an instance whose Ez became NaN or Inf."""
        out = np.zeros(len(self.instances), dtype=np.uint32)
        _lib.check(self.lib.pc_batch_instance_status(self.h, out.ctypes.data_as(C.POINTER(C.c_uint32)),
                                                     self.stream.cuda_stream), "pc_batch_instance_status")
        return out

    # -- results ------------------------------------------------------------------
    def spectra(self):
        """Per instance, per port: complex128 (nf, n) DFT of Ez on the port line."""
        _lib.check(self.lib.pc_batch_dft_flush(self.h, self.stream.cuda_stream), "pc_batch_dft_flush")
        self.stream.synchronize()
        acc = self.acc.double().cpu().numpy()
        z = (acc[..., 0] - acc[..., 2]) + 1j * (acc[..., 1] - acc[..., 3])
        out = []
        pos = 0
        for I in self.instances:
            row = []
            for p in I.ports:
                row.append(z[:, pos:pos + p.n])
                pos += p.n
            out.append(row)
        return out

    def fields(self, q: int):
        """(Ez, Hx, Hy) of instance q as reference-shaped device views."""
        nx, ny = self.instances[q].eps.shape
        f_off, pitch = self.offsets[q][0], self.offsets[q][1]
        s = self.sets[self.cur]
        blk = s[f_off:f_off + 3 * nx * pitch].view(3, nx, pitch)
        return blk[0, : nx - 1, : ny - 1], blk[1, : nx - 1, :ny], blk[2, :nx, : ny - 1]

    def close(self):
        if getattr(self, "h", None):
            self.lib.pc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class SweepResult:
    designs: List[CouplerDesign]
    layouts: List[CouplerLayout]
    S: np.ndarray  # (nd, 4, nf) complex
    seconds: float
    cell_steps: int
    launches: int = 0
    variant: int = -1
    run_seconds: float = 0.0
    rerun: List[int] = field(default_factory=list)   # designs re-run on the per-simulation path
    failed: List[int] = field(default_factory=list)  # designs that failed there too (S is NaN)

    @property
    def designs_per_s(self) -> float:
        return len(self.designs) / self.seconds


def batched_sweep(designs: Sequence[CouplerDesign], nsteps: int = STEPS, nfreq: int = NFREQ, device=None,
                  autotune: bool = True, layouts=None, variant: Optional[int] = None,
                  prepare: Optional[Callable[["BatchedFDTD2D"], None]] = None) -> SweepResult:
    """S-parameters of every design from one batched run (couplers + normalisations).

    ``seconds`` runs from the design list to the S-parameters (layouts, device
    setup, time loop, spectra); ``run_seconds`` is the time loop and spectra.
    ``prepare`` (optional) is called with the batch before the time loop, e.g. to
    seed initial fields.  A design whose coupler or normalisation instance ends
    with a non-finite field is re-run on the per-simulation path
    (``serial_sweep``) and listed in ``rerun``; if it fails there as well its
    S-parameters are NaN and it is listed in ``failed`` (the reference's sweep
    marks such a point as an error and goes on, optimization/sweep.py:183-195)."""
    import torch

    dev = torch.device(device or "cuda")
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    layouts = layouts or [coupler_layout(d) for d in designs]
    freqs = sweep_freqs(nfreq)
    B = BatchedFDTD2D(instances_for(layouts), freqs, device=dev, autotune=autotune, variant=variant)
    try:
        if prepare is not None:
            prepare(B)
        torch.cuda.synchronize(B.device)
        l0 = B.launches
        t1 = time.perf_counter()
        B.run(nsteps)
        spec = B.spectra()
        st = B.instance_status()
        t2 = time.perf_counter()
        bad = [q for q in range(len(layouts)) if (st[2 * q] | st[2 * q + 1]) & _lib.PC_STATUS_NONFINITE]
        S = np.stack([s_parameters(spec[2 * q], spec[2 * q + 1][0], L) if q not in bad
                      else np.full((4, len(freqs)), np.nan + 0j) for q, L in enumerate(layouts)])
        failed = []
        for q in bad:
            try:
                S[q] = serial_sweep([designs[q]], nsteps=nsteps, nfreq=nfreq, device=dev, layouts=[layouts[q]],
                                    warm=False).S[0]
            except FloatingPointError:
                failed.append(q)
        t3 = time.perf_counter()
        cells = sum(I.eps.shape[0] * I.eps.shape[1] for I in B.instances) * nsteps
        r = SweepResult(list(designs), list(layouts), S, t3 - t0, cells, B.launches - l0, B.tuning()[0])
        r.run_seconds = t2 - t1
        r.rerun, r.failed = bad, failed
        return r
    finally:
        B.close()


def serial_sweep(designs: Sequence[CouplerDesign], nsteps: int = STEPS, nfreq: int = NFREQ, device=None,
                 layouts=None, warm: bool = True, batch_route: bool = True) -> SweepResult:
    """The plain path: one single-simulation 2D engine per coupler and per
    normalisation run, one after another (ParameterSweep's sequential loop).
    Timed like ``batched_sweep``: from the design list to the S-parameters.
    ``batch_route``: the engine's 2D batched route (K steps per launch) or its
    per-step kernels."""
    import torch

    from .engine import FDTDEngine

    dev = torch.device(device or "cuda")
    if warm:  # one short untimed run: library load, first-launch and allocator warm-up
        serial_sweep(designs[:1], nsteps=16, nfreq=nfreq, device=device, warm=False, batch_route=batch_route)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    layouts = layouts or [coupler_layout(d) for d in designs]
    freqs = sweep_freqs(nfreq)
    dt = sweep_dt()
    amps = amplitudes(nsteps, dt)[:, None]
    S = []
    cells = 0
    launches = 0
    for L in layouts:
        spec = []
        for eps, ports in ((L.eps, L.ports), (L.norm_eps, L.ports[:1])):
            nx, ny = eps.shape
            eng = FDTDEngine((nx, ny, 1), (DX, DX, DX), dt, is_2d=True, precision="fp32",
                             material_arrays={"eps_rel": eps[:, :, None]}, pml=PMLParams(CPML), device=dev,
                             batch_route=batch_route)
            idx = (np.array([[L.src.x]]), np.arange(L.src.y0, L.src.y0 + L.src.n)[None, :])
            eng.add_source("Ez", eng.offsets("Ez", idx), L.src.profile, None)
            ids = []
            for p in ports:
                pidx = (np.array([[p.x]]), np.arange(p.y0, p.y0 + p.n)[None, :])
                ids.append(eng.add_dft("Ez", eng.offsets("Ez", pidx), freqs, dt))
            eng.step(nsteps, amps)
            try:
                eng.check_status()
            except FloatingPointError:
                eng.close()
                raise
            spec.append([eng.dft_result(m).cpu().numpy().reshape(len(freqs), -1) for m in ids])
            launches += eng.launch_count()
            cells += nx * ny * nsteps
            eng.close()
        S.append(s_parameters(spec[0], spec[1][0], L))
    torch.cuda.synchronize(dev)
    dt_s = time.perf_counter() - t0
    return SweepResult(list(designs), list(layouts), np.stack(S), dt_s, cells, launches)
