"""Mode ports (boundaries/mode_port.py:1-580): inject waveguide modes into, and
extract their coefficients from, device fields.

The port plane, its index bounds (``int()`` of the offset from the grid origin,
mode_port.py:125-205) and the mode profiles interpolated onto it
(RegularGridInterpolator, zero outside, utils/mode_matching.py:358-420) are
restated on the host.  ``inject_fields`` adds Re(A exp(i w t)) times the real
profile to the port's tangential E and normal H components (mode_port.py:261-365)
with the native scatter-add (float64 sum rounded once, as NumPy's in-place add);
``extract_mode_coefficients`` forms a_m = 1/2 sum (E x H_m* + E_m* x H)_n dA / P_m
(utils/mode_matching.py:41-171 with the port's spacing, mode_port.py:367-429) as
one native weighted reduction over the plane.  Fields are this package's
ElectromagneticFields (device arrays); like the reference, ports need a 3D grid.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import _lib

# components added by the injection (mode_port.py:327-365) and the terms of the
# overlap's normal Poynting component (S_n = F0 F1 - F2 F3)
_INJECT = {"x": ("Ey", "Ez", "Hx"), "y": ("Ex", "Ez", "Hy"), "z": ("Ex", "Ey", "Hz")}
_TERMS = {"x": ("Ey", "Hz", "Ez", "Hy"), "y": ("Ez", "Hx", "Ex", "Hz"), "z": ("Ex", "Hy", "Ey", "Hx")}
_COMPS = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")


@dataclass
class ModePortConfig:
    """mode_port.py:22-44."""

    center: tuple
    size: tuple
    direction: str
    modes: list
    inject: bool = False


class _Mode:
    """A mode profile on the port plane (the fields WaveguideMode carries)."""

    def __init__(self, src, fields):
        for k in ("mode_number", "neff", "frequency", "wavelength"):
            setattr(self, k, getattr(src, k, None))
        for c, v in fields.items():
            setattr(self, c, v)


def interpolate_mode(mode, u: np.ndarray, v: np.ndarray) -> _Mode:
    """utils/mode_matching.py:358-420: each 2D component bilinearly interpolated
    from (mode.x, mode.y) to the grid (u, v), zero outside; other components zero."""
    from scipy.interpolate import RegularGridInterpolator

    U, V = np.meshgrid(u, v, indexing="ij")
    pts = np.column_stack([U.ravel(), V.ravel()])
    out = {}
    for c in _COMPS:
        a = np.asarray(getattr(mode, c))
        if a.ndim != 2:
            out[c] = np.zeros((len(u), len(v)), dtype=complex)
            continue
        re = RegularGridInterpolator((mode.x, mode.y), a.real, bounds_error=False, fill_value=0.0)(pts)
        im = RegularGridInterpolator((mode.x, mode.y), a.imag, bounds_error=False, fill_value=0.0)(pts)
        out[c] = (re + 1j * im).reshape(U.shape)
    return _Mode(mode, out)


class ModePort:
    """mode_port.py:47-580 on device fields."""

    def __init__(self, config: ModePortConfig, name: Optional[str] = None, enabled: bool = True):
        self.config = config
        self.name = name or f"ModePort_{id(self)}"
        self.enabled = enabled
        self._grid = None
        self._port_region = {}
        self._interpolated_modes: List[_Mode] = []
        self._mode_coefficients = {i: [] for i in range(len(config.modes))}
        self._time_points: list = []
        self.sign = +1 if config.direction[0] == "+" else -1
        self.axis = config.direction[-1].lower()
        self._dev = {}
        self.lib = None

    # -- setup -------------------------------------------------------------------
    def initialize(self, grid) -> None:
        if not grid.is_3d:
            raise ValueError("mode ports index fields as [x, y, z]: a 3D grid is required")
        self._grid = grid
        self._setup_port_region()
        self._interpolate_modes()
        self._dev = {}

    def _setup_port_region(self) -> None:
        g, c, s = self._grid, self.config.center, self.config.size
        o = g.origin
        lo = lambda a, d: int((c[a] - s[a] / 2 - o[a]) / d)  # noqa: E731
        hi = lambda a, d: int((c[a] + s[a] / 2 - o[a]) / d)  # noqa: E731
        at = lambda a, d: int((c[a] - o[a]) / d)  # noqa: E731
        if self.axis == "x":
            self._port_region = {"x_idx": at(0, g.dx), "y_slice": slice(lo(1, g.dy), hi(1, g.dy)),
                                 "z_slice": slice(lo(2, g.dz), hi(2, g.dz)), "normal_axis": 0}
        elif self.axis == "y":
            self._port_region = {"x_slice": slice(lo(0, g.dx), hi(0, g.dx)), "y_idx": at(1, g.dy),
                                 "z_slice": slice(lo(2, g.dz), hi(2, g.dz)), "normal_axis": 1}
        else:
            self._port_region = {"x_slice": slice(lo(0, g.dx), hi(0, g.dx)), "y_slice": slice(lo(1, g.dy), hi(1, g.dy)),
                                 "z_idx": at(2, g.dz), "normal_axis": 2}

    def _transverse(self):
        r, g = self._port_region, self._grid
        if self.axis == "x":
            return (np.arange(r["y_slice"].start, r["y_slice"].stop) * g.dy + g.origin[1],
                    np.arange(r["z_slice"].start, r["z_slice"].stop) * g.dz + g.origin[2])
        if self.axis == "y":
            return (np.arange(r["x_slice"].start, r["x_slice"].stop) * g.dx + g.origin[0],
                    np.arange(r["z_slice"].start, r["z_slice"].stop) * g.dz + g.origin[2])
        return (np.arange(r["x_slice"].start, r["x_slice"].stop) * g.dx + g.origin[0],
                np.arange(r["y_slice"].start, r["y_slice"].stop) * g.dy + g.origin[1])

    def _interpolate_modes(self) -> None:
        u, v = self._transverse()
        self._interpolated_modes = [interpolate_mode(m, u, v) for m in self.config.modes]

    def _index(self):
        r = self._port_region
        if self.axis == "x":
            return (r["x_idx"], r["y_slice"], r["z_slice"])
        if self.axis == "y":
            return (r["x_slice"], r["y_idx"], r["z_slice"])
        return (r["x_slice"], r["y_slice"], r["z_idx"])

    def _offsets(self, view, shape_only=False):
        """Element offsets of the port plane inside a component view (from its strides)."""
        idx = self._index()
        axes = []
        for a, ix in enumerate(idx):
            n = view.shape[a]
            axes.append(np.array([ix]) if isinstance(ix, (int, np.integer)) else np.arange(n)[ix])
        st = view.stride()
        grids = np.meshgrid(*axes, indexing="ij")
        off = sum(gx.astype(np.int64) * st[a] for a, gx in enumerate(grids))
        return off.reshape(-1) if not shape_only else off.shape

    # -- device helpers ----------------------------------------------------------------
    def _lib(self):
        if self.lib is None:
            self.lib = _lib.load()
        return self.lib

    @staticmethod
    def _view(fields, comp):
        x = fields[comp]
        return getattr(x, "tensor", x)

    def _stream(self, t):
        import torch

        return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)

    # -- injection ----------------------------------------------------------------------
    def inject_fields(self, fields, time: float, dt: float, mode_amplitudes=None) -> None:
        """Add Re(A exp(i w t)) times each mode's real profile (mode_port.py:261-365)."""
        import torch

        if not self.enabled or not self.config.inject:
            return
        if mode_amplitudes is None:
            mode_amplitudes = [1.0] * len(self._interpolated_modes)
        lib = self._lib()
        for m, (mode, amp) in enumerate(zip(self._interpolated_modes, mode_amplitudes)):
            amp_real = (amp * np.exp(1j * (2 * np.pi * mode.frequency * time))).real
            for comp in _INJECT[self.axis]:
                view = self._view(fields, comp)
                key = ("inj", m, comp, view.dtype)
                if key not in self._dev:
                    off = self._offsets(view)
                    w = np.asarray(getattr(mode, comp)).real.reshape(-1)
                    if w.size != off.size:
                        raise ValueError(f"{comp}: mode profile has {w.size} points, port plane {off.size}")
                    self._dev[key] = (torch.as_tensor(off, device=view.device),
                                      torch.as_tensor(np.ascontiguousarray(w, dtype=np.float64), device=view.device))
                d_off, d_w = self._dev[key]
                _lib.check(lib.pc_scatter_add(8 if view.dtype == torch.float64 else 4, view.data_ptr(),
                                              d_off.data_ptr(), d_w.data_ptr(), d_off.numel(), float(amp_real),
                                              self._stream(view)), "pc_scatter_add")

    # -- extraction --------------------------------------------------------------------
    def _spacing(self):
        g = self._grid
        dx = g.dx if self.axis != "x" else g.dy
        dy = g.dy if self.axis != "y" else (g.dz if g.is_3d else g.dx)
        return dx, dy

    def _weights(self, npts):
        """[nmodes][4][npts] complex: 1/2 dA / P_m times the overlap's profile factors."""
        dx, dy = self._spacing()
        f0, f1, f2, f3 = _TERMS[self.axis]
        w = np.zeros((len(self._interpolated_modes), 4, npts), dtype=np.complex128)
        for m, md in enumerate(self._interpolated_modes):
            a = {c: np.asarray(getattr(md, c)) for c in _COMPS}
            s = a[f0] * np.conj(a[f1]) - a[f2] * np.conj(a[f3])
            p = float(abs(0.5 * np.real(np.sum(s)) * dx * dy))  # compute_mode_power
            if abs(p) <= 1e-20:
                continue  # compute_mode_overlap returns 0
            k = 0.5 * dx * dy / p
            w[m, 0] = k * np.conj(a[f1]).reshape(-1)
            w[m, 1] = k * a[f0].reshape(-1)
            w[m, 2] = -k * np.conj(a[f3]).reshape(-1)
            w[m, 3] = -k * a[f2].reshape(-1)
        return w

    def extract_mode_coefficients(self, fields, time: float):
        """Mode coefficients of the current fields (mode_port.py:367-429)."""
        import torch

        if not self.enabled:
            return [0.0] * len(self._interpolated_modes)
        terms = _TERMS[self.axis]
        views = [self._view(fields, c) for c in terms]
        key = ("ext", views[0].dtype)
        if key not in self._dev:
            offs = [self._offsets(v) for v in views]
            npts = offs[0].size
            if any(o.size != npts for o in offs):
                raise ValueError("port plane differs between components")
            w = self._weights(npts)
            self._dev[key] = (torch.as_tensor(np.concatenate(offs), device=views[0].device),
                              torch.as_tensor(np.ascontiguousarray(np.stack([w.real, w.imag], -1).reshape(-1)),
                                              device=views[0].device), npts)
        d_off, d_w, npts = self._dev[key]
        nm = len(self._interpolated_modes)
        out = torch.zeros(2 * nm, dtype=torch.float64, device=views[0].device)
        P = C.c_void_p * 4
        _lib.check(self._lib().pc_plane_overlap(8 if views[0].dtype == torch.float64 else 4,
                                                P(*[v.data_ptr() for v in views]), d_off.data_ptr(), int(npts),
                                                int(nm), d_w.data_ptr(), out.data_ptr(), self._stream(views[0])),
                   "pc_plane_overlap")
        o = out.cpu().numpy()
        coeffs = [complex(o[2 * m], o[2 * m + 1]) for m in range(nm)]
        for m, c in enumerate(coeffs):
            self._mode_coefficients[m].append(c)
        self._time_points.append(time)
        return coeffs

    def get_mode_coefficient(self, mode_index: int):
        return self._mode_coefficients[mode_index]

    def get_time_points(self):
        return self._time_points
