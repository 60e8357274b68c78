"""Sources with the reference's interface (sources/*.py), injected on the device.

Each source resolves its index region exactly as the reference does
(``Source._setup_source_region``, sources/base.py:62-139) and, when attached to
a cuda simulation, registers a device-side soft source
``field[idx] += weight * a(t_{n+1})`` that the stepping kernels apply after the
E update of each step (sources/point.py:62-73, sources/plane_wave.py:184-221).
The host only evaluates the scalar waveform a(t) in float64.
"""

from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Callable, Optional, Sequence

import numpy as np


# ---------------------------------------------------------------------------
# waveforms (sources/waveform.py)
# ---------------------------------------------------------------------------
class Waveform:
    """sources/waveform.py:14-60."""

    def __init__(self, amplitude: float = 1.0, phase: float = 0.0):
        self.amplitude = amplitude
        self.phase = phase

    def __call__(self, t):
        return self.evaluate(t)

    def evaluate(self, t):
        raise NotImplementedError("Subclasses must implement evaluate method")


class ContinuousWave(Waveform):
    """sources/waveform.py:63-96: A sin(w t + phi)."""

    def __init__(self, frequency: float, amplitude: float = 1.0, phase: float = 0.0):
        super().__init__(amplitude, phase)
        self.frequency = frequency
        self.omega = 2 * np.pi * frequency

    def evaluate(self, t):
        return self.amplitude * np.sin(self.omega * t + self.phase)


class GaussianPulse(Waveform):
    """sources/waveform.py:99-152: A exp(-tau^2/2) sin(w t + phi), tau = (t - delay)/width,
    delay defaulting to 3 widths."""

    def __init__(self, frequency: float, pulse_width: float, amplitude: float = 1.0, phase: float = 0.0,
                 delay: Optional[float] = None):
        super().__init__(amplitude, phase)
        self.frequency = frequency
        self.pulse_width = pulse_width
        self.omega = 2 * np.pi * frequency
        self.delay = delay if delay is not None else 3 * pulse_width

    def evaluate(self, t):
        tau = (t - self.delay) / self.pulse_width
        envelope = np.exp(-0.5 * tau * tau)
        return self.amplitude * envelope * np.sin(self.omega * t + self.phase)


class CustomWaveform(Waveform):
    """A user callable a(t)."""

    def __init__(self, func: Callable, amplitude: float = 1.0):
        super().__init__(amplitude, 0.0)
        self.func = func

    def evaluate(self, t):
        return self.amplitude * self.func(t)


# ---------------------------------------------------------------------------
# sources
# ---------------------------------------------------------------------------
def _identity(a):
    return a


def _per_z0(a):  # gaussian.py:262-266: H carries a / 377
    return a / 377.0


class Source(ABC):
    """sources/base.py:17-150 (same constructor and region semantics)."""

    def __init__(self, center, size, name: Optional[str] = None, enabled: bool = True):
        self.center = center
        self.size = size
        self.name = name or f"{self.__class__.__name__}_{id(self)}"
        self.enabled = enabled
        self._grid = None
        self._source_region = {}

    def initialize(self, grid) -> None:
        self._grid = grid
        self._setup_source_region()

    def _setup_source_region(self) -> None:
        if self._grid is None:
            raise RuntimeError("Source must be initialized with a grid first")
        b = self._grid.region_bounds(self.center, self.size)
        self._source_region = {c: self._grid.get_component_indices(c, *b)
                               for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")}

    def _compute_source_region(self):
        if self._grid is None:
            raise RuntimeError("Source must be initialized with a grid first")
        return self._grid.region_bounds(self.center, self.size)

    @abstractmethod
    def injections(self):
        """List of (component, index tuple, weight array or None, amp_fn): the device
        applies field[idx] += weight * amp_fn(a(t)) every step.  amp_fn reproduces
        the reference's float64 expression for the added amplitude."""

    def amplitude(self, t):
        return self.waveform(t)

    def update_fields(self, fields, time: float, dt: float) -> None:
        """Host path for fields that are not bound to a device engine."""
        if not self.enabled:
            return
        a = self.amplitude(time)
        for comp, idx, w, fn in self.injections():
            f = fields[comp]
            f[idx] += fn(a) if w is None else (w * fn(a))


class PointSource(Source):
    """sources/point.py:14-73."""

    def __init__(self, position, component: str, waveform: Waveform, name: Optional[str] = None,
                 enabled: bool = True):
        super().__init__(center=position, size=(0, 0, 0), name=name, enabled=enabled)
        self.component = component
        self.waveform = waveform

    def injections(self):
        return [(self.component, self._source_region[self.component], None, _identity)]


class ElectricDipole(PointSource):
    """sources/point.py:76-140."""

    def __init__(self, position, polarization: str, frequency: float, pulse: bool = True,
                 pulse_width: Optional[float] = None, amplitude: float = 1.0, phase: float = 0.0,
                 name: Optional[str] = None, enabled: bool = True):
        component = {"x": "Ex", "y": "Ey", "z": "Ez"}[polarization.lower()]
        if pulse:
            if pulse_width is None:
                raise ValueError("pulse_width must be provided for pulsed sources")
            wf = GaussianPulse(frequency=frequency, pulse_width=pulse_width, amplitude=amplitude, phase=phase)
        else:
            wf = ContinuousWave(frequency=frequency, amplitude=amplitude, phase=phase)
        super().__init__(position=position, component=component, waveform=wf, name=name, enabled=enabled)


class MagneticDipole(PointSource):
    """sources/point.py (magnetic counterpart): H component soft source."""

    def __init__(self, position, polarization: str, frequency: float, pulse: bool = True,
                 pulse_width: Optional[float] = None, amplitude: float = 1.0, phase: float = 0.0,
                 name: Optional[str] = None, enabled: bool = True):
        component = {"x": "Hx", "y": "Hy", "z": "Hz"}[polarization.lower()]
        if pulse:
            if pulse_width is None:
                raise ValueError("pulse_width must be provided for pulsed sources")
            wf = GaussianPulse(frequency=frequency, pulse_width=pulse_width, amplitude=amplitude, phase=phase)
        else:
            wf = ContinuousWave(frequency=frequency, amplitude=amplitude, phase=phase)
        super().__init__(position=position, component=component, waveform=wf, name=name, enabled=enabled)


class PlaneWaveSource(Source):
    """sources/plane_wave.py:17-221: E += a*sign, H += a/377*sign over the region."""

    _MAP = {("x", "y"): ("Ey", "Hz"), ("x", "z"): ("Ez", "Hy"), ("y", "x"): ("Ex", "Hz"),
            ("y", "z"): ("Ez", "Hx"), ("z", "x"): ("Ex", "Hy"), ("z", "y"): ("Ey", "Hx")}

    def __init__(self, center, size, direction: str, polarization: str, frequency: float,
                 pulse: bool = True, pulse_width: Optional[float] = None, amplitude: float = 1.0,
                 phase: float = 0.0, name: Optional[str] = None, enabled: bool = True):
        super().__init__(center=center, size=size, name=name, enabled=enabled)
        if direction.startswith("+"):
            self.direction, self.direction_sign = direction[1:], 1
        elif direction.startswith("-"):
            self.direction, self.direction_sign = direction[1:], -1
        else:
            self.direction, self.direction_sign = direction, 1
        if self.direction.lower() not in ("x", "y", "z"):
            raise ValueError(f"Invalid direction: {direction}. Must be one of: x, y, z, +x, -x, +y, -y, +z, -z")
        if self.direction.lower() == polarization.lower():
            raise ValueError(f"Polarization ({polarization}) must be perpendicular to propagation direction "
                             f"({direction})")
        self.polarization = polarization
        self.frequency = frequency
        if pulse:
            if pulse_width is None:
                raise ValueError("pulse_width must be provided for pulsed sources")
            self.waveform = GaussianPulse(frequency, pulse_width, amplitude, phase)
        else:
            self.waveform = ContinuousWave(frequency, amplitude, phase)

    def injections(self):
        e, h = self._MAP[(self.direction.lower(), self.polarization.lower())]
        s = self.direction_sign
        # plane_wave.py:211-221: E += a * sign, H += (a / 377) * sign
        return [(e, self._source_region[e], None, lambda a: a * s),
                (h, self._source_region[h], None, lambda a: (a / 377.0) * s)]


class LineSource(Source):
    """Soft source over a region with a per-point profile (a sampled mode shape):
    field[idx] += profile * a(t).  ``profile`` has the region's shape for the
    component, or is None for a uniform line."""

    def __init__(self, center, size, component: str, waveform: Waveform, profile: Optional[np.ndarray] = None,
                 name: Optional[str] = None, enabled: bool = True):
        super().__init__(center=center, size=size, name=name, enabled=enabled)
        self.component = component
        self.waveform = waveform
        self.profile = None if profile is None else np.asarray(profile, dtype=np.float64)

    def injections(self):
        idx = self._source_region[self.component]
        w = None
        if self.profile is not None:
            shape = tuple(np.asarray(i).size for i in idx)
            w = np.broadcast_to(self.profile.reshape(-1) if self.profile.size == int(np.prod(shape))
                                else self.profile, (int(np.prod(shape)),)).reshape(shape)
        return [(self.component, idx, w, _identity)]


class GaussianBeamSource(Source):
    """sources/gaussian.py:18-298: on the source region, E += a(t) exp(-r^2/w0^2) and
    H += a(t) exp(-r^2/w0^2) / 377 with r the transverse distance of each region
    point from the beam centre (the reference's profile of _calculate_beam_profile,
    160-268, over the region's index ranges; each component's index set takes the
    profile values in C order, as ``field[indices] += values.flat`` does)."""

    _MAP = PlaneWaveSource._MAP

    def __init__(self, center, size, direction: str, polarization: str, frequency: float, beam_waist: float,
                 pulse: bool = True, pulse_width: Optional[float] = None, amplitude: float = 1.0,
                 phase: float = 0.0, name: Optional[str] = None, enabled: bool = True):
        super().__init__(center=center, size=size, name=name, enabled=enabled)
        if direction.lower() == polarization.lower():
            raise ValueError(f"Polarization ({polarization}) must be perpendicular to propagation direction "
                             f"({direction})")
        if (direction.lower(), polarization.lower()) not in self._MAP:
            raise ValueError(f"Invalid direction ({direction}) and polarization ({polarization}) combination")
        self.direction = direction
        self.polarization = polarization
        self.frequency = frequency
        self.beam_waist = beam_waist
        if pulse:
            if pulse_width is None:
                raise ValueError("pulse_width must be provided for pulsed sources")
            self.waveform = GaussianPulse(frequency, pulse_width, amplitude, phase)
        else:
            self.waveform = ContinuousWave(frequency, amplitude, phase)

    def beam_profile(self) -> np.ndarray:
        """exp(-r^2 / w0^2) on the region's transverse index grid (no time factor)."""
        g = self._grid
        x0, x1, y0, y1, z0, z1 = self._compute_source_region()
        is3d = getattr(g, "is_3d", len(g.dimensions) == 3 and g.dimensions[2] > 1)
        if not is3d and z0 == z1:
            z1 = z0 + 1
        d = self.direction.lower()
        if d == "x":
            ys, zs = np.meshgrid(np.arange(y0, y1), np.arange(z0, z1), indexing="ij")
            r2 = (g.index_to_coord(1, ys) - self.center[1]) ** 2
            if is3d:
                r2 = r2 + (g.index_to_coord(2, zs) - self.center[2]) ** 2
        elif d == "y":
            xs, zs = np.meshgrid(np.arange(x0, x1), np.arange(z0, z1), indexing="ij")
            r2 = (g.index_to_coord(0, xs) - self.center[0]) ** 2
            if is3d:
                r2 = r2 + (g.index_to_coord(2, zs) - self.center[2]) ** 2
        else:
            xs, ys = np.meshgrid(np.arange(x0, x1), np.arange(y0, y1), indexing="ij")
            r2 = (g.index_to_coord(0, xs) - self.center[0]) ** 2 + (g.index_to_coord(1, ys) - self.center[1]) ** 2
        return np.exp(-r2 / self.beam_waist**2)

    def injections(self):
        e, h = self._MAP[(self.direction.lower(), self.polarization.lower())]
        prof = self.beam_profile().ravel()
        out = []
        for comp, fn in ((e, _identity), (h, _per_z0)):
            idx = self._source_region[comp]
            shape = tuple(np.asarray(i).size for i in idx)
            n = int(np.prod(shape))
            if prof.size != n:
                raise ValueError(f"beam profile has {prof.size} values for {n} {comp} points of the region")
            out.append((comp, idx, prof.reshape(shape), fn))
        return out


class ModeSource(Source):
    """sources/mode.py:19-361: a waveguide mode injected on a plane.  The mode's
    transverse field profiles (real parts, already sampled on the source plane's
    points of each component: ``profiles = {component: array}``) are added with
    the amplitude A w(t) cos(phase - omega t) (update_fields, 198-253: the real part
    of A w(t) exp(i(phase - omega t))); the normal H component takes the
    propagation sign (+x/-x, ...)."""

    def __init__(self, center, size, profiles: dict, direction: str, waveform: Waveform, frequency: float,
                 amplitude: float = 1.0, phase: float = 0.0, name: Optional[str] = None, enabled: bool = True):
        super().__init__(center=center, size=size, name=name, enabled=enabled)
        if direction[0] not in "+-" or direction[-1].lower() not in "xyz":
            raise ValueError("direction must be one of +x, -x, +y, -y, +z, -z")
        self.direction = direction
        self.sign = +1 if direction[0] == "+" else -1
        self.axis = direction[-1].lower()
        self.profiles = {c: np.asarray(v, dtype=np.float64) for c, v in profiles.items()}
        self.waveform = waveform
        self.frequency = frequency
        self.amplitude_scale = amplitude
        self.phase = phase

    def _normal_h(self) -> str:
        return {"x": "Hx", "y": "Hy", "z": "Hz"}[self.axis]

    def injections(self):
        out = []
        for comp, prof in self.profiles.items():
            idx = self._source_region[comp]
            shape = tuple(np.asarray(i).size for i in idx)
            if prof.size != int(np.prod(shape)):
                raise ValueError(f"{comp} profile has {prof.size} values for {int(np.prod(shape))} points")
            w = prof.reshape(shape) * (self.sign if comp == self._normal_h() else 1.0)
            out.append((comp, idx, w, _identity))
        return out

    def mode_amplitude(self, t):
        """A w(t) cos(phase - omega t) at simulation time t."""
        omega = 2 * np.pi * self.frequency
        return self.amplitude_scale * np.asarray(self.waveform(t)) * np.cos(self.phase - omega * np.asarray(t))

    def amplitude(self, t):
        return self.mode_amplitude(t)


class TFSFSource(Source):
    """Plane-wave total-field/scattered-field source (sources/tfsf.py:17-411
    interface).  On the device it is a consistent TFSF plane fed by a 1D auxiliary
    Yee line (pc_set_tfsf); the plane is the z-index of ``center`` and propagation
    is along +z or -z (the reference's entry-plane correction is replaced)."""

    def __init__(self, center, size, direction: str, polarization: str, frequency: float, pulse: bool = True,
                 pulse_width: Optional[float] = None, amplitude: float = 1.0, phase: float = 0.0,
                 eps_background: float = 1.0, name: Optional[str] = None, enabled: bool = True):
        super().__init__(center=center, size=size, name=name, enabled=enabled)
        sign = -1 if direction.startswith("-") else 1
        axis = direction.lstrip("+-").lower()
        if axis != "z":
            raise NotImplementedError("the device TFSF plane propagates along z")
        if polarization.lower() not in ("x", "y"):
            raise ValueError("polarization must be x or y for z propagation")
        self.direction, self.direction_sign = axis, sign
        self.polarization = polarization.lower()
        self.frequency = frequency
        self.wavelength = 299792458.0 / frequency
        self.eps_background = eps_background
        if pulse:
            if pulse_width is None:
                raise ValueError("pulse_width must be provided for pulsed sources")
            self.waveform = GaussianPulse(frequency, pulse_width, amplitude, phase)
        else:
            self.waveform = ContinuousWave(frequency, amplitude, phase)

    def plane_index(self) -> int:
        return self._grid.point_to_index(self.center)[2]

    def injections(self):
        return []

    def update_fields(self, fields, time, dt):
        raise NotImplementedError("the TFSF plane runs inside the device stepper")


def amplitude_table(sources: Sequence[Source], times: np.ndarray) -> np.ndarray:
    """[len(times), n_injections] amplitudes (disabled sources contribute 0)."""
    cols = []
    for s in sources:
        a = np.asarray(s.amplitude(times), dtype=np.float64) if s.enabled else np.zeros(len(times))
        a = np.broadcast_to(a, (len(times),))
        for _, _, _, fn in s.injections():
            cols.append(np.broadcast_to(fn(a), (len(times),)))
    if not cols:
        return np.zeros((len(times), 0))
    return np.stack(cols, axis=1)
