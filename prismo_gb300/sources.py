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
        a = self.waveform(time)
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
        a = np.asarray(s.waveform(times), dtype=np.float64) if s.enabled else np.zeros(len(times))
        a = np.broadcast_to(a, (len(times),))
        for _, _, _, fn in s.injections():
            cols.append(np.broadcast_to(fn(a), (len(times),)))
    if not cols:
        return np.zeros((len(times), 0))
    return np.stack(cols, axis=1)
