"""Register the "cuda" backend inside the reference Prismo package.

``register()`` wraps, from outside, the registry functions of
backends/backend_manager.py (set_backend 139-186, get_backend 189-241,
list_available_backends 33-67) so that "cuda" is accepted, and makes the
reference classes FDTDSolver, MaxwellUpdater (core/solver.py:24, 571),
ElectromagneticFields (core/fields.py:20) and Simulation (core/simulation.py:22)
construct this package's native versions while the cuda backend is selected
(their ``__new__`` is wrapped, which also covers every module that imported the
classes by name).  Reference sources and monitors passed to a cuda Simulation
are mapped to device injections / device DFT monitors over the same index
regions.  No reference file is modified; with any other backend the reference
code runs unchanged.
"""

from __future__ import annotations

import importlib
from typing import Optional

_state = {"registered": False}


def _cuda_backend_class(ref_base):
    from .backend import CudaBackend

    class RefCudaBackend(CudaBackend, ref_base):
        """The cuda backend, also an instance of the reference Backend ABC."""

    return RefCudaBackend


def register(prismo_module=None) -> None:
    """Install the "cuda" backend into an importable ``prismo`` package."""
    if _state["registered"]:
        return
    prismo = prismo_module or importlib.import_module("prismo")
    bm = importlib.import_module("prismo.backends.backend_manager")
    base = importlib.import_module("prismo.backends.base")
    from . import backend as nb

    RefCuda = _cuda_backend_class(base.Backend)
    orig_set, orig_get, orig_list = bm.set_backend, bm.get_backend, bm.list_available_backends

    def list_available_backends():
        names = list(orig_list())
        if "cuda" in nb.list_available_backends():
            names.append("cuda")
        return names

    def set_backend(backend: str, device_id: int = 0, **kwargs):
        if backend.lower() == "cuda":
            if "cuda" not in nb.list_available_backends():
                raise ValueError("cuda backend requested but no CUDA device is available")
            b = RefCuda(device_id=device_id, **kwargs)
            bm._CURRENT_BACKEND = b
            nb._CURRENT = b
            return b
        nb._CURRENT = None
        return orig_set(backend, device_id)

    def get_backend(backend: Optional[str] = None, device_id: int = 0, **kwargs):
        if backend is not None:
            return set_backend(backend, device_id, **kwargs)
        return orig_get(None, device_id)

    for mod in (bm, importlib.import_module("prismo.backends"), prismo):
        if hasattr(mod, "set_backend"):
            mod.set_backend = set_backend
        if hasattr(mod, "get_backend"):
            mod.get_backend = get_backend
        if hasattr(mod, "list_available_backends"):
            mod.list_available_backends = list_available_backends

    def cuda_selected(kwargs) -> bool:
        b = kwargs.get("backend")
        if isinstance(b, str):
            return b.lower() == "cuda"
        if b is not None:
            return getattr(b, "name", None) == "cuda"
        return getattr(bm._CURRENT_BACKEND, "name", None) == "cuda"

    from . import fields as nf
    from . import solver as ns

    def reroute(ref_cls, native_cls, adapt=None):
        def __new__(cls, *args, **kwargs):
            if cls is ref_cls and cuda_selected(kwargs):
                if adapt is not None:
                    args, kwargs = adapt(args, kwargs)
                if "backend" in kwargs and not isinstance(kwargs["backend"], (str, nb.Backend, type(None))):
                    kwargs["backend"] = "cuda"
                return native_cls(*args, **kwargs)
            return object.__new__(cls)

        ref_cls.__new__ = __new__

    solver_mod = importlib.import_module("prismo.core.solver")
    fields_mod = importlib.import_module("prismo.core.fields")
    sim_mod = importlib.import_module("prismo.core.simulation")
    reroute(solver_mod.FDTDSolver, ns.FDTDSolver)
    reroute(solver_mod.MaxwellUpdater, ns.MaxwellUpdater)
    reroute(fields_mod.ElectromagneticFields, nf.ElectromagneticFields)
    reroute(sim_mod.Simulation, AdaptingSimulation)
    _state["registered"] = True


class AdaptingSimulation:
    """Factory used for reference ``Simulation(...)`` calls under the cuda backend:
    returns a native Simulation whose add_source / add_monitor also accept the
    reference's source and monitor objects."""

    def __new__(cls, *args, **kwargs):
        from .simulation import Simulation

        sim = Simulation(*args, **kwargs)
        native_add_source, native_add_monitor = sim.add_source, sim.add_monitor

        def add_source(source):
            native_add_source(_adapt_source(source))

        def add_monitor(monitor):
            native_add_monitor(_adapt_monitor(monitor))

        sim.add_source = add_source
        sim.add_monitor = add_monitor
        return sim


def _adapt_source(src):
    """Reference source -> this package's source with the same region and waveform."""
    from . import sources as S

    if isinstance(src, S.Source):
        return src
    name = type(src).__name__
    if hasattr(src, "component") and hasattr(src, "waveform") and name in ("PointSource", "ElectricDipole",
                                                                          "MagneticDipole"):
        out = S.PointSource(position=src.center, component=src.component, waveform=src.waveform, name=src.name,
                            enabled=src.enabled)
        return out
    if name == "PlaneWaveSource":
        out = S.PlaneWaveSource.__new__(S.PlaneWaveSource)
        S.Source.__init__(out, center=src.center, size=src.size, name=src.name, enabled=src.enabled)
        out.direction, out.direction_sign = src.direction, src.direction_sign
        out.polarization = src.polarization
        out.frequency = getattr(src, "frequency", None)
        out.waveform = src.waveform
        return out
    if name == "GaussianBeamSource":
        out = S.GaussianBeamSource.__new__(S.GaussianBeamSource)
        S.Source.__init__(out, center=src.center, size=src.size, name=src.name, enabled=src.enabled)
        out.direction, out.polarization = src.direction, src.polarization
        out.frequency, out.beam_waist = src.frequency, src.beam_waist
        out.waveform = src.waveform
        return out
    return src  # unknown type: applied from the host on device arrays


def _adapt_monitor(mon):
    from . import monitors as M

    if isinstance(mon, M.Monitor):
        return mon
    name = type(mon).__name__
    if name == "FieldMonitor":
        out = M.FieldMonitor(center=mon.center, size=mon.size, components=list(mon.components), name=mon.name,
                             time_domain=mon.time_domain, frequencies=list(mon.frequencies))
        _mirror(mon, out)
        return out
    if name == "DFTMonitor":
        out = M.DFTMonitor(center=mon.center, size=mon.size, frequencies=list(mon.frequencies),
                           components=list(mon.components), name=mon.name)
        _mirror(mon, out)
        return out
    if name == "ModeExpansionMonitor":
        out = M.ModeExpansionMonitor(center=mon.center, size=mon.size, modes=list(mon.modes), direction=mon.direction,
                                     frequencies=None if mon.frequencies is None else list(mon.frequencies),
                                     name=mon.name)
        _mirror(mon, out)
        return out
    if name == "FluxMonitor":
        out = M.FluxMonitor(center=mon.center, size=mon.size, direction=mon.direction, name=mon.name,
                            frequencies=None if mon.frequencies is None else list(mon.frequencies))
        _mirror(mon, out)
        return out
    raise TypeError(f"monitor type {name} is not supported by the cuda backend")


def _mirror(ref, native):
    """Route the reference monitor's accessors to the device monitor."""
    for attr in ("get_time_data", "get_frequency_data", "get_power_flow", "get_intensity", "get_power_spectrum",
                 "get_time_domain_power", "get_frequency_domain_power", "get_transmission", "get_mode_coefficient",
                 "separate_forward_backward", "get_mode_power", "get_mode_transmission", "compute_s_parameters",
                 "update", "initialize"):
        if hasattr(native, attr):
            setattr(ref, attr, getattr(native, attr))
    ref._native = native
