"""Device-side FDTD engine: one libprismo_cuda context plus its device buffers.

Field storage (one allocation per set): a tensor of shape (6, nx, ny, pitch) in
3D or (6, nx, pitch) in 2D, component order Ex, Ey, Ez, Hx, Hy, Hz, fast axis
padded to a multiple of 32 elements (128 B rows in float32).  Each component's
reference-shaped array (core/grid.py:157-168) is a strided view of its slab;
the padding stays zero.  The fused 3D schedule alternates between two such
sets (reads set ``cur``, writes ``cur ^ 1``); the split schedule updates one
set in place.

Coefficients are built on the device from cell-centred material arrays
(core/solver.py:113-133, 458-533) and kept in the same padded layout: Cb per E
component always, Ca only when some sigma_e != 0, Da/Db arrays only when
mu_rel != 1 or sigma_m != 0 (otherwise the scalars 1 and dt/mu0).
"""

from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .pml import PMLParams, cpml_axis_coefficients

EPS0 = 8.854187817e-12
MU0 = 4 * np.pi * 1e-7
COMPONENTS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
COMP_INDEX = {c: i for i, c in enumerate(COMPONENTS)}


def _torch():
    import torch

    return torch


def component_shape(comp: str, dims, is_2d: bool):
    """core/grid.py:157-168."""
    nx, ny, nz = dims
    if is_2d:
        return {"Ex": (nx, ny - 1), "Ey": (nx - 1, ny), "Ez": (nx - 1, ny - 1),
                "Hx": (nx - 1, ny), "Hy": (nx, ny - 1), "Hz": (nx, ny)}[comp]
    return {"Ex": (nx, ny - 1, nz - 1), "Ey": (nx - 1, ny, nz - 1), "Ez": (nx - 1, ny - 1, nz),
            "Hx": (nx - 1, ny, nz), "Hy": (nx, ny - 1, nz), "Hz": (nx, ny, nz - 1)}[comp]


def new_field_sets(buf_shape, dtype, device, n):
    torch = _torch()
    return [torch.zeros(buf_shape, dtype=dtype, device=device) for _ in range(n)]


def storage_shape(dims, is_2d: bool):
    """Padded field-set shape: (6, nx, pitch) in 2D, (6, nx, ny, pitch) in 3D."""
    nx, ny, nz = dims
    if is_2d:
        return (6, nx, _round_up(ny, 32))
    return (6, nx, ny, _round_up(nz, 32))


def torch_complex(re, im):
    torch = _torch()
    return torch.complex(re, im)


def _round_up(x: int, m: int) -> int:
    return (x + m - 1) // m * m


class FDTDEngine:
    """Owns a native stepping context; see module docstring for the layout."""

    def __init__(self, dims: Sequence[int], spacing: Sequence[float], dt: float, *, is_2d: bool,
                 precision: str = "fp32", mode: str = "corrected", sched: str = "auto",
                 material_arrays: Optional[dict] = None, pml: Optional[PMLParams] = None,
                 device: Optional[str] = None, stream=None, sets=None, bind_later: bool = False,
                 batch_route: bool = True):
        torch = _torch()
        self.lib = _lib.load()
        if not torch.cuda.is_available():
            raise RuntimeError("the cuda backend needs a CUDA device")
        # default: the current device (a replica per GPU sets it from LOCAL_RANK).  The
        # library allocates and launches on the current device, so it must be this one.
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        if self.device.index is not None and self.device.index != torch.cuda.current_device():
            raise ValueError(f"FDTDEngine on {self.device} while cuda:{torch.cuda.current_device()} is current; "
                             "make it current first (torch.cuda.set_device)")
        self.is_2d = bool(is_2d)
        nx, ny, nz = (int(d) for d in dims)
        if self.is_2d:
            nz = 1
        self.dims = (nx, ny, nz)
        self.spacing = tuple(float(s) for s in spacing)
        self.dt = float(dt)
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.precision = precision
        self.dtype = torch.float32 if precision == "fp32" else torch.float64
        self.mode = {"corrected": _lib.PC_MODE_CORRECTED, "legacy": _lib.PC_MODE_LEGACY}[mode]
        self.sched = {"auto": _lib.PC_SCHED_AUTO, "split": _lib.PC_SCHED_SPLIT,
                      "fused": _lib.PC_SCHED_FUSED}[sched]
        fast = ny if self.is_2d else nz
        self.pitch = _round_up(fast, 32)
        self.buf_shape = (6, nx, self.pitch) if self.is_2d else (6, nx, ny, self.pitch)
        self.stream = stream if stream is not None else torch.cuda.current_stream(self.device)

        desc = _lib.GridDesc()
        desc.ndim = 2 if self.is_2d else 3
        desc.nx, desc.ny, desc.nz = nx, ny, nz
        desc.pitch = self.pitch
        desc.precision = 4 if precision == "fp32" else 8
        desc.mode = self.mode
        desc.sched = self.sched
        desc.dt = self.dt
        desc.dx, desc.dy = self.spacing[0], self.spacing[1]
        desc.dz = self.spacing[2] if not self.is_2d else 0.0
        self.desc = desc
        ctx = C.c_void_p()
        _lib.check(self.lib.pc_create(C.byref(desc), C.byref(ctx)), "pc_create")
        self.ctx = ctx
        # the library resolves AUTO; ping-pong sets are needed for the fused 3D schedule
        self.pingpong = (not self.is_2d) and self.mode == _lib.PC_MODE_CORRECTED and \
            self.sched in (_lib.PC_SCHED_AUTO, _lib.PC_SCHED_FUSED)
        self.sets = []
        if not bind_later:
            if sets is None:
                sets = new_field_sets(self.buf_shape, self.dtype, self.device, 2 if self.pingpong else 1)
            self.bind(sets, 0)
        self._set_materials(material_arrays)
        self.pml = None
        self.psi = []
        if pml is not None and int(pml.thickness) > 0:
            self._set_cpml(pml)
        self.sources = []  # (comp, offsets, weights, waveform)
        self.dfts = []  # (comp, offsets, omegas, accumulator tensor)
        self.fluxes = []  # per-step power histories (device float64)
        self.mode_mons = []  # per-step mode-coefficient histories (device complex128)
        self._dft_t0 = []
        # 2D TE simulations of the shape the batched kernel covers run on it (see _route_2d)
        self.batch_route = bool(batch_route)
        self._route = None
        self._stepped = False
        self._closed = False

    # -- setup ---------------------------------------------------------------
    def bind(self, sets, cur: int = 0):
        """Attach field storage: a list of one or two tensors of shape buf_shape
        (a second set is allocated when the schedule ping-pongs)."""
        sets = list(sets)
        for t in sets:
            if tuple(t.shape) != tuple(self.buf_shape) or t.dtype != self.dtype or not t.is_contiguous():
                raise ValueError(f"field storage must be contiguous {self.dtype} of shape {self.buf_shape}")
        if self.pingpong and len(sets) < 2:
            sets.append(new_field_sets(self.buf_shape, self.dtype, self.device, 1)[0])
            if cur == 1:
                raise ValueError("current set 1 without a second set")
        self.sets = sets
        s0 = _lib.P6(*[sets[0][q].data_ptr() for q in range(6)])
        s1 = _lib.P6(*[sets[1][q].data_ptr() for q in range(6)]) if self.pingpong else None
        _lib.check(self.lib.pc_set_fields(self.ctx, s0, s1), "pc_set_fields")
        if cur:
            _lib.check(self.lib.pc_set_current_set(self.ctx, int(cur)), "pc_set_current_set")

    def _set_materials(self, ma: Optional[dict]):
        torch = _torch()
        ma = ma or {}
        nx, ny, nz = self.dims
        cell_shape = (nx, ny, nz)

        def dev(name):
            v = ma.get(name)
            if v is None:
                return None
            if isinstance(v, torch.Tensor):
                t = v.to(device=self.device, dtype=torch.float64).contiguous()
            else:
                t = torch.as_tensor(np.ascontiguousarray(np.asarray(v, dtype=np.float64)), device=self.device)
            if tuple(t.shape) != cell_shape:
                raise ValueError(f"{name} must have shape {cell_shape}, got {tuple(t.shape)}")
            return t

        eps, mu, sig, sigm = dev("eps_rel"), dev("mu_rel"), dev("sigma_e"), dev("sigma_m")
        self._eps_cells = eps  # the cell permittivity (device, float64), for the 2D batched route
        need_ca = sig is not None and bool(torch.any(sig != 0).item())
        need_h = (mu is not None and bool(torch.any(mu != 1).item())) or \
                 (sigm is not None and bool(torch.any(sigm != 0).item()))
        ncoef = 3 + (3 if need_ca else 0) + (6 if need_h else 0)
        shape = (ncoef,) + self.buf_shape[1:]
        self.coef = torch.empty(shape, dtype=self.dtype, device=self.device)
        cb = [self.coef[q] for q in range(3)]
        ca = [self.coef[3 + q] for q in range(3)] if need_ca else [None] * 3
        base = 3 + (3 if need_ca else 0)
        da = [self.coef[base + q] for q in range(3)] if need_h else [None] * 3
        db = [self.coef[base + 3 + q] for q in range(3)] if need_h else [None] * 3
        sp = self._stream_ptr()
        ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        _lib.check(self.lib.pc_build_coefficients(
            # all-zero sigma (or mu = 1, sigma_m = 0) arrays give the same bits as none
            self.ctx, ptr(eps), ptr(mu) if need_h else None, ptr(sig) if need_ca else None,
            ptr(sigm) if need_h else None, EPS0, MU0,
            _lib.ptr3(ca) if need_ca else None, _lib.ptr3(cb),
            _lib.ptr3(da) if need_h else None, _lib.ptr3(db) if need_h else None, sp),
            "pc_build_coefficients")
        # scalar H coefficients for mu_rel = 1, sigma_m = 0 (core/solver.py:129-131)
        db_s = (self.dt / (MU0 * 1.0)) / (1.0 + 0.0)
        _lib.check(self.lib.pc_set_coefficients(
            self.ctx, _lib.ptr3(ca) if need_ca else None, _lib.ptr3(cb),
            _lib.ptr3(da) if need_h else None, _lib.ptr3(db) if need_h else None, 1.0, db_s),
            "pc_set_coefficients")
        self.has_ca, self.has_hcoef = need_ca, need_h
        self._mat_refs = (eps, mu, sig, sigm)  # keep alive until the build kernel ran
        self.synchronize()
        self._mat_refs = None

    def _set_cpml(self, params: PMLParams):
        torch = _torch()
        t = int(params.thickness)
        nx, ny, nz = self.dims
        d_max = max(self.spacing[:2] if self.is_2d else self.spacing)
        ns = [nx, ny] + ([] if self.is_2d else [nz])
        prof = [cpml_axis_coefficients(n, params, d_max, self.dt) for n in ns]
        self._cpml_host = prof  # keep the float64 arrays alive during the call
        arrs = [[np.ascontiguousarray(p[w]) for p in prof] for w in range(3)]
        D = C.POINTER(C.c_double)
        mk = lambda lst: _lib.D3(*([x.ctypes.data_as(D) for x in lst] + [None] * (3 - len(lst))))  # noqa: E731
        nel = int(self.lib.pc_cpml_psi_elems(C.byref(self.desc), t))
        self.psi = [torch.zeros(nel, dtype=self.dtype, device=self.device)]
        if self.pingpong:
            self.psi.append(torch.zeros(nel, dtype=self.dtype, device=self.device))
        _lib.check(self.lib.pc_set_cpml(self.ctx, t, mk(arrs[0]), mk(arrs[1]), mk(arrs[2]),
                                        self.psi[0].data_ptr(),
                                        self.psi[1].data_ptr() if self.pingpong else None), "pc_set_cpml")
        self.pml = params

    # -- access --------------------------------------------------------------
    def _stream_ptr(self):
        return self.stream.cuda_stream

    @property
    def cur(self) -> int:
        if self._route is not None:
            return self._route.cur
        return int(self.lib.pc_current_set(self.ctx))

    def component(self, comp: str, set_index: Optional[int] = None):
        """Reference-shaped view (core/grid.py:157-168) of a component."""
        q = COMP_INDEX[comp]
        s = self.sets[self.cur if set_index is None else set_index]
        shp = component_shape(comp, self.dims, self.is_2d)
        if self.is_2d:
            return s[q, : shp[0], : shp[1]]
        return s[q, : shp[0], : shp[1], : shp[2]]

    def offsets(self, comp: str, index) -> np.ndarray:
        """Flat element offsets (padded layout) of a reference index tuple."""
        shp = component_shape(comp, self.dims, self.is_2d)
        grid = np.zeros(shp, dtype=bool)
        grid[index] = True
        idx = np.nonzero(grid)
        if self.is_2d:
            return (idx[0].astype(np.int64) * self.pitch + idx[1]).astype(np.int64)
        ny = self.dims[1]
        return ((idx[0].astype(np.int64) * ny + idx[1]) * self.pitch + idx[2]).astype(np.int64)

    # -- sources ---------------------------------------------------------------
    def add_source(self, comp: str, offsets: np.ndarray, weights: Optional[np.ndarray], waveform) -> int:
        offs = np.ascontiguousarray(offsets, dtype=np.int64)
        w = None if weights is None else np.ascontiguousarray(np.broadcast_to(weights, offs.shape), dtype=np.float64)
        sid = _lib.check(self.lib.pc_add_source(
            self.ctx, COMP_INDEX[comp], offs.ctypes.data_as(C.POINTER(C.c_int64)),
            None if w is None else w.ctypes.data_as(C.POINTER(C.c_double)), int(offs.size)), "pc_add_source")
        self.sources.append((comp, offs, w, waveform))
        self._route_check("add_source")
        return sid

    # -- dispersive regions ----------------------------------------------------------
    def set_dispersive(self, regions):
        """Dispersive (ADE) regions: a list of (box, eps_inf, poles) with box =
        (x0, x1, y0, y1, z0, z1) in each E component's own index space and poles
        dicts from ``prismo_gb300.materials`` (kind lorentz/drude/debye with C0..C3).
        Allocates the zeroed auxiliary arrays on the device."""
        torch = _torch()
        kinds = {"lorentz": 0, "drude": 1, "debye": 2}
        arr = (_lib.AdeRegion * max(1, len(regions)))()
        self.ade_aux = []
        for r, (box, eps_inf, poles) in enumerate(regions):
            R = arr[r]
            box = [int(b) for b in box]
            if self.is_2d:
                box = box[:4] + [0, 1]
            for q in range(6):
                R.box[q] = box[q]
            R.npoles = len(poles)
            R.eps_inf = float(eps_inf)
            shape = (box[1] - box[0], box[3] - box[2], box[5] - box[4])
            for pi, p in enumerate(poles):
                R.kind[pi] = kinds[p["kind"]]
                R.c0[pi], R.c1[pi] = float(p["C0"]), float(p["C1"])
                R.c2[pi], R.c3[pi] = float(p.get("C2", 0.0)), float(p.get("C3", 0.0))
                for c in range(3):
                    for w in range(2 if p["kind"] == "lorentz" else 1):
                        t = torch.zeros(shape, dtype=self.dtype, device=self.device)
                        self.ade_aux.append(t)
                        R.aux[c][pi][w] = t.data_ptr()
        _lib.check(self.lib.pc_set_ade(self.ctx, len(regions), arr, EPS0), "pc_set_ade")
        self.ade_regions = regions

    # -- TFSF plane ------------------------------------------------------------------
    def set_tfsf(self, k0: int, direction: int, polarization: str, waveform, eps_b: float = 1.0, m0: int = 4,
                 max_steps: int = 20000):
        """Plane-wave TFSF injection at z-plane k0 (see pc_set_tfsf); the auxiliary
        line is long enough that its far-end reflection cannot reach the sample
        point within ``max_steps`` steps."""
        import math

        C0_ = 299792458.0
        m = m0 + int(math.ceil(0.5 * max_steps * C0_ * self.dt / self.spacing[2])) + 8
        _lib.check(self.lib.pc_set_tfsf(self.ctx, int(k0), int(direction), 0 if polarization == "x" else 1,
                                        int(m0), int(m), float(eps_b), EPS0), "pc_set_tfsf")
        self.tfsf = waveform

    # -- DFT monitors ------------------------------------------------------------
    def add_dft(self, comp: str, offsets: np.ndarray, freqs, t0: float) -> int:
        """Device DFT running sum of ``comp`` at ``offsets`` for ``freqs`` (Hz); the
        first sample is taken after the next step, at simulation time ``t0``."""
        torch = _torch()
        offs = np.ascontiguousarray(offsets, dtype=np.int64)
        om = np.ascontiguousarray(2 * np.pi * np.asarray(freqs, dtype=np.float64))
        acc = torch.zeros((len(om), offs.size, 4), dtype=torch.float32, device=self.device)
        mid = _lib.check(self.lib.pc_add_dft(
            self.ctx, COMP_INDEX[comp], offs.ctypes.data_as(C.POINTER(C.c_int64)), int(offs.size),
            om.ctypes.data_as(C.POINTER(C.c_double)), int(om.size), self.dt, float(t0), acc.data_ptr()),
            "pc_add_dft")
        self.dfts.append((comp, offs, om, acc))
        self._dft_t0.append(float(t0))
        self._route_check("add_dft")
        return mid

    def dft_result(self, mid: int):
        """Complex (nf, npts) accumulator of a DFT monitor (flushes pending samples)."""
        if self._route is not None:
            torch = _torch()
            return torch.as_tensor(self._route.spectra()[0][mid], device=self.device)
        _lib.check(self.lib.pc_dft_flush(self.ctx, int(mid), self._stream_ptr()), "pc_dft_flush")
        acc = self.dfts[mid][3].double()
        return torch_complex(acc[..., 0] - acc[..., 2], acc[..., 1] - acc[..., 3])

    # -- flux monitors -----------------------------------------------------------
    def add_flux(self, comps, offsets, scale: float, capacity: int = 1 << 18) -> int:
        """Per-step power sum_p (F0 F1 - F2 F3)(p) * scale through a plane, F0..F3
        the components ``comps`` at ``offsets`` [4][npts]; returns the monitor id."""
        torch = _torch()
        offs = np.ascontiguousarray(offsets, dtype=np.int64).reshape(4, -1)
        cs = (C.c_int32 * 4)(*[COMP_INDEX[c] for c in comps])
        hist = torch.zeros(int(capacity), dtype=torch.float64, device=self.device)
        fid = _lib.check(self.lib.pc_add_flux(self.ctx, cs, offs.ctypes.data_as(C.POINTER(C.c_int64)),
                                              int(offs.shape[1]), float(scale), hist.data_ptr(), int(capacity)),
                         "pc_add_flux")
        self.fluxes.append(hist)
        return fid

    def flux_history(self, fid: int) -> np.ndarray:
        """Power of every step sampled so far by flux monitor ``fid`` (float64)."""
        n = C.c_int64(0)
        _lib.check(self.lib.pc_flux_count(self.ctx, int(fid), C.byref(n), self._stream_ptr()), "pc_flux_count")
        hist = self.fluxes[fid]
        if n.value > hist.numel():
            raise RuntimeError(f"flux monitor {fid}: {n.value} steps sampled, history holds {hist.numel()}")
        return hist[:n.value].cpu().numpy()

    def flux_spectrum(self, dft_ids, scale: float) -> np.ndarray:
        """1/2 Re sum_p (F0 F1* - F2 F3*) * scale from the DFT monitors ``dft_ids``."""
        torch = _torch()
        nf = self.dfts[dft_ids[0]][2].size
        out = torch.zeros(nf, dtype=torch.float64, device=self.device)
        ids = (C.c_int32 * 4)(*[int(i) for i in dft_ids])
        _lib.check(self.lib.pc_flux_spectrum(self.ctx, ids, float(scale), out.data_ptr(), self._stream_ptr()),
                   "pc_flux_spectrum")
        return out.cpu().numpy()

    # -- mode-expansion monitors ------------------------------------------------
    def add_mode_monitor(self, comps, offsets, weights, capacity: int = 1 << 16) -> int:
        """Per-step complex a_m = sum_q,p weights[m][q][p] F_q(offsets[q][p]) for every
        mode m (weights complex [nmodes][4][npts]); returns the monitor id."""
        torch = _torch()
        offs = np.ascontiguousarray(offsets, dtype=np.int64).reshape(4, -1)
        w = np.asarray(weights, dtype=np.complex128)
        nm = w.shape[0]
        wr = np.ascontiguousarray(np.stack([w.real, w.imag], axis=-1).reshape(-1))
        cs = (C.c_int32 * 4)(*[COMP_INDEX[c] for c in comps])
        hist = torch.zeros((int(capacity), nm), dtype=torch.complex128, device=self.device)
        mid = _lib.check(self.lib.pc_add_mode_monitor(
            self.ctx, cs, offs.ctypes.data_as(C.POINTER(C.c_int64)), int(offs.shape[1]), int(nm),
            wr.ctypes.data_as(C.POINTER(C.c_double)), hist.data_ptr(), int(capacity)), "pc_add_mode_monitor")
        self.mode_mons.append(hist)
        return mid

    def mode_history(self, mid: int) -> np.ndarray:
        """[steps][nmodes] complex coefficients sampled so far."""
        n = C.c_int64(0)
        _lib.check(self.lib.pc_mode_count(self.ctx, int(mid), C.byref(n), self._stream_ptr()), "pc_mode_count")
        hist = self.mode_mons[mid]
        if n.value > hist.shape[0]:
            raise RuntimeError(f"mode monitor {mid}: {n.value} steps sampled, history holds {hist.shape[0]}")
        return hist[:n.value].cpu().numpy()

    def mode_spectrum(self, mid: int, freqs, t0: float) -> np.ndarray:
        """[nmodes][nf] sum_n a_m(t_n) exp(-i w t_n) dt, t_n = t0 + n dt."""
        torch = _torch()
        om = np.ascontiguousarray(2 * np.pi * np.asarray(freqs, dtype=np.float64))
        nm = self.mode_mons[mid].shape[1]
        out = torch.zeros((nm, om.size), dtype=torch.complex128, device=self.device)
        _lib.check(self.lib.pc_mode_spectrum(self.ctx, int(mid), om.ctypes.data_as(C.POINTER(C.c_double)),
                                             int(om.size), float(t0), float(self.dt), out.data_ptr(),
                                             self._stream_ptr()), "pc_mode_spectrum")
        return out.cpu().numpy()

    # -- stepping --------------------------------------------------------------
    def step(self, nsteps: int = 1, amps: Optional[np.ndarray] = None):
        """Advance nsteps; amps[nsteps, nsources] are the source amplitudes at
        t_{n+1} of each step (sources/point.py:62-73)."""
        if self._route is None and not self._stepped and self.batch_route:
            self._route = self._route_2d()
        self._stepped = True
        if self._route is not None:
            self._route.step(int(nsteps), amps)
            return
        ns = len(self.sources) + (1 if getattr(self, "tfsf", None) is not None else 0)
        ap = None
        if ns:
            a = np.ascontiguousarray(amps, dtype=np.float64).reshape(nsteps, ns)
            self._amps_keep = a
            ap = a.ctypes.data_as(C.POINTER(C.c_double))
        _lib.check(self.lib.pc_step(self.ctx, int(nsteps), ap, self._stream_ptr()), "pc_step")

    def status(self) -> int:
        v = C.c_uint32(0)
        _lib.check(self.lib.pc_status(self.ctx, C.byref(v), self._stream_ptr()), "pc_status")
        return int(v.value) | (self._route.status() if self._route is not None else 0)

    # -- the 2D batched route ------------------------------------------------------
    def _route_2d(self):
        """A one-instance batched run (csrc/batch.cu: K time steps per launch in
        shared memory) of this engine's own Ez, Hx, Hy buffers, when the
        simulation has the shape that kernel covers: 2D, float32, corrected
        stepper, lossless non-magnetic media, dx = dy, the default CPML profile,
        at most one soft Ez source on one x column over consecutive y, at most
        four Ez DFT lines of that form sharing their frequencies and first sample
        time, no flux or mode monitors, and the Hz family (Ex, Ey, Hz) zero.
        Decided at the first step; returns None when the shape does not fit."""
        if not (self.is_2d and self.precision == "fp32" and self.mode == _lib.PC_MODE_CORRECTED):
            return None
        if self.has_ca or self.has_hcoef or getattr(self, "tfsf", None) is not None or self.fluxes or \
                self.mode_mons or getattr(self, "ade_aux", None):
            return None
        if self.spacing[0] != self.spacing[1] or len(self.sources) > 1 or len(self.dfts) > 4:
            return None
        t = 0 if self.pml is None else int(self.pml.thickness)
        if self.pml is not None and self.pml != PMLParams(thickness=t):
            return None
        if any(float(self.component(c).abs().max()) != 0.0 for c in ("Ex", "Ey", "Hz")):
            return None

        def line(offs):
            x, y = offs // self.pitch, offs % self.pitch
            if offs.size == 0 or np.any(x != x[0]) or np.any(y != y[0] + np.arange(offs.size)):
                return None
            return int(x[0]), int(y[0]), int(offs.size)

        from . import sweep as SW

        if self.sources:
            comp, offs, w, _ = self.sources[0]
            ln = line(offs)
            if comp != "Ez" or ln is None:
                return None
            src = SW.Port(ln[0], ln[1], ln[2], np.ones(ln[2]) if w is None else np.asarray(w, dtype=np.float64))
        else:
            src = SW.Port(1, 1, 0, np.zeros(0))
        ports = []
        for q, (comp, offs, om, _) in enumerate(self.dfts):
            ln = line(offs)
            if comp != "Ez" or ln is None or not np.array_equal(om, self.dfts[0][2]) or \
                    self._dft_t0[q] != self._dft_t0[0]:
                return None
            ports.append(SW.Port(ln[0], ln[1], ln[2], np.ones(ln[2])))
        nx, ny = self.dims[0], self.dims[1]
        if nx < 2 * t + 4 or ny < 2 * t + 4:
            return None
        eps = self._eps_cells
        eps = np.ones((nx, ny)) if eps is None else eps.reshape(nx, ny).double().cpu().numpy()
        torch = _torch()
        # the batch steps components 2-4 (Ez, Hx, Hy) of the engine's set buffers
        # in place, ping-pong between them: a second set joins the engine's
        if len(self.sets) < 2:
            self.sets.append(torch.zeros_like(self.sets[0]))
        freqs = self.dfts[0][2] / (2 * np.pi) if self.dfts else np.array([1.0])
        # one instance, 4 steps per pass, without timing every variant: 32 x 64 tiles,
        # or 32 x 32 when 32 x 64 leaves fewer than two tiles per SM (a single 500 x 250
        # grid: 64 tiles of 32 x 64 for 152 SMs; its batch runs at 19.1 Gcell/s on
        # 32 x 32 tiles against 14.3 on 32 x 64, the variant the tuner then picks too)
        nx_, ny_ = eps.shape
        sms = torch.cuda.get_device_properties(self.device).multi_processor_count
        small = -(-nx_ // 32) * -(-ny_ // 64) < 2 * sms
        want = (32, 32, 4) if small else (32, 64, 4)
        variant = next((v for v, tv in enumerate(SW.BatchedFDTD2D.variants()) if tuple(tv) == want), 1)
        return _Route2D(self, SW.BatchedFDTD2D(
            [SW.Instance(np.ascontiguousarray(eps), src, ports)], freqs, dx=self.spacing[0], dt=self.dt, cpml=t,
            device=self.device, stream=self.stream, field_sets=[s_[2:5] for s_ in self.sets[:2]],
            dft_t0=self._dft_t0[0] if self.dfts else None, autotune=False, variant=variant))

    def _route_check(self, what):
        if self._route is not None:
            raise RuntimeError(f"{what} after the first step of a simulation on the 2D batched route; "
                               "create the engine with batch_route=False to change it between steps")

    def check_status(self):
        st = self.status()
        if st & _lib.PC_STATUS_BOUNDS:
            raise IndexError("a kernel computed an out-of-range auxiliary-array offset (skipped)")
        if st & _lib.PC_STATUS_TIMEOUT:
            raise TimeoutError("a bounded device wait ran out inside the FDTD kernel")
        if st & _lib.PC_STATUS_NONFINITE:
            raise FloatingPointError("non-finite field values detected")
        return st

    def profile(self, enable: bool = True):
        _lib.check(self.lib.pc_profile(self.ctx, 1 if enable else 0), "pc_profile")

    def profile_read(self):
        """(summed ms, launches, time steps) of the main stencil kernel since the
        last read (a launch of the temporally blocked stepper covers two steps)."""
        ms = C.c_double(0)
        n = C.c_int64(0)
        steps = int(self.lib.pc_profile_steps(self.ctx))
        _lib.check(self.lib.pc_profile_read(self.ctx, C.byref(ms), C.byref(n)), "pc_profile_read")
        return float(ms.value), int(n.value), steps

    def set_time_blocking(self, steps: int, chunk: int = 0, order: Optional[int] = None):
        """Time steps per launch of the temporally blocked 3D stepper (2: two steps
        per launch wherever no monitor samples the step in between, 1: one, 0:
        off, the fused schedule runs), its x-chunk length (0: automatic) and its
        work-item order (0 grid order, 1 expensive chunks first, 2 by item cost)."""
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_TS_STEPS, int(steps)), "pc_set_tuning")
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_TS_CHUNK, int(chunk)), "pc_set_tuning")
        if order is not None:
            _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_TS_ORDER, int(order)), "pc_set_tuning")

    def time_blocking(self):
        return (int(self.lib.pc_get_tuning(self.ctx, _lib.PC_TUNE_TS_STEPS)),
                int(self.lib.pc_get_tuning(self.ctx, _lib.PC_TUNE_TS_CHUNK)),
                int(self.lib.pc_get_tuning(self.ctx, _lib.PC_TUNE_TS_ORDER)))

    def time_blocking_active(self) -> bool:
        """Whether the temporally blocked stepper runs for this configuration."""
        return bool(self.lib.pc_get_tuning(self.ctx, _lib.PC_TUNE_TS_ACTIVE))

    # -- autotuning ---------------------------------------------------------------
    def autotune(self, candidates=(8, 16, 24, 32, 48, 64, 96), steps: int = 20, cache: bool = True):
        """Pick the x-chunk lengths of the 3D schedule by timing a few steps of each
        candidate with CUDA events.  Fused schedule: first one length for every
        tile, then, with that fixed for the inner tiles, the length for tiles that
        touch a y or z CPML slab; returns (chunk, edge chunk).  Temporally blocked
        stepper: every pair of chunk length and work-item order; returns (chunk,
        order).  The fields and psi are restored afterwards.  Results are cached
        per (dims, CPML thickness, precision, schedule) in ``$PRISMO_GB300_CACHE``
        (default ~/.cache/prismo_gb300/tune.json)."""
        import json
        import os

        torch = _torch()
        if self.is_2d or not self.pingpong:
            return None
        blocked = self.time_blocking_active()
        if not blocked and (getattr(self, "ade_aux", None) or getattr(self, "tfsf", None) is not None or self.dfts
                            or self.fluxes or self.mode_mons):
            # ADE auxiliaries, the TFSF line and monitor sums would advance with the
            # timed steps: time a plain engine of the same grid on the same kernels
            # (the chunk choice does not depend on those extras' few per-point terms)
            if self.has_ca or self.has_hcoef:
                return None
            shadow = FDTDEngine(self.dims, self.spacing, self.dt, is_2d=False, precision=self.precision,
                                sched="fused", pml=self.pml, device=str(self.device), stream=self.stream)
            try:
                shadow.set_time_blocking(0)
                res = shadow.autotune(candidates, steps, cache)
            finally:
                shadow.close()
            if res is not None:
                self.set_chunk(*res)
            return res
        key = f"{self.dims}|t={0 if self.pml is None else self.pml.thickness}|{self.precision}|" \
              f"{'ts' if blocked else 'fused'}|{torch.cuda.get_device_name(self.device)}"
        path = os.environ.get("PRISMO_GB300_CACHE", os.path.join(os.path.expanduser("~"), ".cache",
                                                                 "prismo_gb300", "tune.json"))
        table = {}
        if cache and os.path.exists(path):
            try:
                with open(path) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
        if cache and isinstance(table.get(key), list) and len(table[key]) == 2:
            cx, ce = (int(v) for v in table[key])
            if blocked:
                self.set_time_blocking(self.time_blocking()[0], cx, ce)
            else:
                self.set_chunk(cx, ce)
            return cx, ce
        saved_sets = [t.clone() for t in self.sets]
        saved_psi = [t.clone() for t in self.psi]
        saved_cur = self.cur
        nsrc = len(self.sources)
        amps = np.zeros((steps, nsrc)) if nsrc else None

        ts_steps = self.time_blocking()[0]

        def timed(cx, ce):
            if blocked:  # (chunk, work-item order) of the temporally blocked stepper
                self.set_time_blocking(ts_steps, cx, ce)
            else:
                self.set_chunk(cx, ce)
            self.step(2, None if amps is None else amps[:2])
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            self.step(steps, amps)
            e1.record(self.stream)
            e1.synchronize()
            return e0.elapsed_time(e1)

        cands = [c for c in candidates if c < self.dims[0]]
        best, best_ms = None, float("inf")
        best_e = 2 if blocked else 0
        for cx in cands:
            # blocked stepper: every (chunk, order) pair (the best order depends on the
            # chunk: at 256^3, 64 / expensive-first beats 96, the best chunk by cost order)
            for order in ((2, 1, 0) if blocked else (0,)):
                ms = timed(cx, order)
                if ms < best_ms:
                    best, best_e, best_ms = cx, order, ms
        if not blocked and best is not None and self.pml is not None:
            for ce in cands:
                if ce == best:
                    continue
                ms = timed(best, ce)
                if ms < best_ms:
                    best_e, best_ms = ce, ms
        for dst, src in zip(self.sets, saved_sets):
            dst.copy_(src)
        for dst, src in zip(self.psi, saved_psi):
            dst.copy_(src)
        _lib.check(self.lib.pc_set_current_set(self.ctx, saved_cur), "pc_set_current_set")
        self.check_status()
        if best is None:
            return None
        if blocked:
            self.set_time_blocking(ts_steps, best, best_e)
        else:
            self.set_chunk(best, best_e)
        if cache:
            table[key] = [best, best_e]
            try:
                os.makedirs(os.path.dirname(path), exist_ok=True)
                with open(path, "w") as f:
                    json.dump(table, f, indent=1)
            except OSError:
                pass
        return best, best_e

    def set_chunk(self, cx: int, edge: int = 0):
        """x-chunk length of the fused 3D schedule; `edge` for tiles that touch a y
        or z CPML slab (0: the same as cx)."""
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_FUSED_CHUNK, int(cx)), "pc_set_tuning")
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_FUSED_CHUNK_EDGE, int(edge)), "pc_set_tuning")

    def chunk(self) -> int:
        return int(self.lib.pc_get_tuning(self.ctx, _lib.PC_TUNE_FUSED_CHUNK))

    def set_split(self, level: int, unified: Optional[bool] = None):
        """CPML work items with a kernel variant of their own slab axes: 0 none, 1
        items on one axis's slabs, 2 also items on two axes' slabs (default);
        `unified`: all variants in one launch (default) instead of one launch per
        variant on concurrent streams."""
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_FUSED_SPLIT, int(level)), "pc_set_tuning")
        if unified is not None:
            _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_FUSED_UNIFIED, int(bool(unified))),
                       "pc_set_tuning")

    def chunk_edge(self) -> int:
        return int(self.lib.pc_get_tuning(self.ctx, _lib.PC_TUNE_FUSED_CHUNK_EDGE))

    def set_fused_extras(self, on: bool = True):
        """3D grids with ADE regions or a TFSF plane: on the fused schedule (the
        plane corrections and the ADE partial update in the fused H + E kernel, the
        pole terms in one pass per region; default) or on the split kernels."""
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_FUSED_EXTRAS, int(bool(on))), "pc_set_tuning")

    def set_graph_steps(self, n: int):
        """Steps per captured time-loop graph (a multiple of 16; 0 = eager steps)."""
        _lib.check(self.lib.pc_set_tuning(self.ctx, _lib.PC_TUNE_GRAPH_STEPS, int(n)), "pc_set_tuning")

    def launch_count(self) -> int:
        return int(self.lib.pc_launch_count(self.ctx)) + (self._route.launches if self._route is not None else 0)

    def synchronize(self):
        self.stream.synchronize()

    def close(self):
        if self._route is not None:
            self._route.close()
            self._route = None
        if not self._closed and self.ctx:
            try:
                self.synchronize()
            finally:
                self.lib.pc_destroy(self.ctx)
                self.ctx = C.c_void_p()
                self._closed = True

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Route2D:
    """The 2D batched route of an FDTDEngine: a one-instance BatchedFDTD2D on the
    engine's buffers, fed the engine's per-call amplitude rows (the batch indexes
    its amplitude table by the step count since it was set up)."""

    def __init__(self, eng, batch):
        self.eng = eng
        self.B = batch
        eng.psi = list(batch.psi)  # zeroing the engine's psi resets the batch's
        self.amps = np.zeros(0)

    @property
    def cur(self) -> int:
        return self.B.cur

    @property
    def launches(self) -> int:
        return self.B.launches

    def step(self, nsteps, amps):
        done = self.B.steps_done
        col = np.zeros(nsteps) if amps is None or not len(self.eng.sources) else \
            np.asarray(amps, dtype=np.float64).reshape(nsteps, -1)[:, 0]
        self.amps = np.concatenate([self.amps[:done], col])
        self.B.set_amplitudes(self.amps)
        self.B.step(nsteps)

    def spectra(self):
        return self.B.spectra()

    def status(self) -> int:
        return self.B.status()

    def close(self):
        self.B.close()
