"""Dispersive materials with the reference interface (materials/dispersion.py).

``permittivity(omega)`` and ``get_ade_coefficients(dt)`` restate
materials/dispersion.py:156-336; the coefficients feed the device ADE update
(pc_set_ade), whose coupling to E is documented in include/prismo_cuda.h.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import List

import numpy as np


@dataclass
class LorentzPole:
    """materials/dispersion.py:16-36."""

    omega_0: float
    delta_epsilon: float
    gamma: float


@dataclass
class DrudePole:
    omega_p: float
    gamma: float


@dataclass
class DebyePole:
    delta_epsilon: float
    tau: float


class DispersiveMaterial:
    def __init__(self, epsilon_inf: float, name: str = ""):
        self.epsilon_inf = epsilon_inf
        self.name = name

    def ade_poles(self, dt: float) -> list:
        """Pole dicts (kind, C0..C3) for the device ADE update."""
        raise NotImplementedError


class LorentzMaterial(DispersiveMaterial):
    """dispersion.py:156-231 (bilinear C0..C3 with C1 = C0)."""

    def __init__(self, epsilon_inf: float, poles: List[LorentzPole], name: str = ""):
        super().__init__(epsilon_inf, name)
        self.poles = poles

    def permittivity(self, omega):
        eps = self.epsilon_inf * np.ones_like(omega, dtype=complex)
        for p in self.poles:
            eps = eps + p.delta_epsilon * p.omega_0**2 / (p.omega_0**2 - omega**2 - 1j * omega * p.gamma)
        return eps

    def get_ade_coefficients(self, dt: float) -> dict:
        out = {"poles": [], "epsilon_inf": self.epsilon_inf}
        for p in self.poles:
            w0, g, de = p.omega_0, p.gamma, p.delta_epsilon
            denom = 4.0 + 2 * g * dt + w0**2 * dt**2
            c0 = 2 * de * w0**2 * dt**2 / denom
            out["poles"].append({"C0": c0, "C1": c0, "C2": (8.0 - 2 * w0**2 * dt**2) / denom,
                                 "C3": -(4.0 - 2 * g * dt + w0**2 * dt**2) / denom,
                                 "omega_0": w0, "gamma": g, "delta_epsilon": de})
        return out

    def ade_poles(self, dt):
        return [dict(kind="lorentz", **{k: p[k] for k in ("C0", "C1", "C2", "C3")})
                for p in self.get_ade_coefficients(dt)["poles"]]


class DrudeMaterial(DispersiveMaterial):
    """dispersion.py:234-286 (exponential step)."""

    def __init__(self, epsilon_inf: float, omega_p: float, gamma: float, name: str = ""):
        super().__init__(epsilon_inf, name)
        self.omega_p = omega_p
        self.gamma = gamma

    def permittivity(self, omega):
        return self.epsilon_inf - self.omega_p**2 / (omega**2 + 1j * omega * self.gamma)

    def get_ade_coefficients(self, dt: float) -> dict:
        e = np.exp(-self.gamma * dt)
        return {"C0": self.omega_p**2 / self.gamma * (1.0 - e), "C1": e, "omega_p": self.omega_p,
                "gamma": self.gamma, "epsilon_inf": self.epsilon_inf}

    def ade_poles(self, dt):
        c = self.get_ade_coefficients(dt)
        return [{"kind": "drude", "C0": c["C0"], "C1": c["C1"]}]


class DebyeMaterial(DispersiveMaterial):
    """dispersion.py:289-336."""

    def __init__(self, epsilon_inf: float, epsilon_s: float, tau: float, name: str = ""):
        super().__init__(epsilon_inf, name)
        self.epsilon_s = epsilon_s
        self.tau = tau

    def permittivity(self, omega):
        return self.epsilon_inf + (self.epsilon_s - self.epsilon_inf) / (1.0 + 1j * omega * self.tau)

    def get_ade_coefficients(self, dt: float) -> dict:
        e = np.exp(-dt / self.tau)
        return {"C0": (self.epsilon_s - self.epsilon_inf) * (1.0 - e), "C1": e, "tau": self.tau,
                "epsilon_s": self.epsilon_s, "epsilon_inf": self.epsilon_inf}

    def ade_poles(self, dt):
        c = self.get_ade_coefficients(dt)
        return [{"kind": "debye", "C0": c["C0"], "C1": c["C1"]}]


class DrudeLorentzMaterial(DispersiveMaterial):
    """One Drude pole plus Lorentz poles sharing eps_inf (a metal model)."""

    def __init__(self, epsilon_inf: float, omega_p: float, gamma: float, lorentz: List[LorentzPole], name=""):
        super().__init__(epsilon_inf, name)
        self.drude = DrudeMaterial(epsilon_inf, omega_p, gamma)
        self.lorentz = LorentzMaterial(0.0, lorentz)

    def permittivity(self, omega):
        return self.drude.permittivity(omega) + self.lorentz.permittivity(omega)

    def ade_poles(self, dt):
        return self.drude.ade_poles(dt) + self.lorentz.ade_poles(dt)
