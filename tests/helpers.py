"""Helpers shared by several test modules (not tests themselves)."""

import os
import sys

import numpy as np
import pytest

# the reference package: an installed copy under baseline/_ref (travels with the
# repository to GPU machines), or a source tree named by PRISMO_REFERENCE_SRC (the
# directory holding the ``prismo`` package); tests that need it skip without both
INSTALLED = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "baseline", "_ref")
SOURCE_TREES = [os.environ.get("PRISMO_REFERENCE_SRC", ""), INSTALLED]


def import_reference(candidates):
    import builtins
    import types

    for path in candidates:
        if path and os.path.isdir(os.path.join(path, "prismo")):
            builtins.MTLBuffer = object
            pl = types.ModuleType("polars")
            pl.DataFrame = object
            sys.modules.setdefault("polars", pl)
            try:  # a reference dependency absent on some machines; only the sweep uses it
                import tqdm  # noqa: F401
            except ImportError:
                tq = types.ModuleType("tqdm")
                tq.tqdm = lambda it=None, *a, **k: it
                sys.modules["tqdm"] = tq
            if path not in sys.path:
                sys.path.insert(0, path)
            import prismo

            return prismo
    pytest.skip("reference package not available")



def port_modes(rng, n=2):
    """Synthetic waveguide modes on their own (x, y) grid (modes/solver.py:17-53 fields)."""
    from types import SimpleNamespace

    u = np.linspace(0.1e-6, 0.9e-6, 23)
    v = np.linspace(0.05e-6, 0.7e-6, 17)
    U, V = np.meshgrid(u, v, indexing="ij")
    out = []
    for k in range(n):
        g = np.exp(-((U - 0.5e-6) ** 2 + (V - 0.35e-6) ** 2) / (0.15e-6) ** 2)
        f = {c: g * (rng.uniform(0.5, 1.5) + 1j * rng.uniform(-0.5, 0.5)) for c in ("Ex", "Ey", "Ez")}
        f.update({c: g * (rng.uniform(-0.01, 0.01) + 1j * rng.uniform(-0.01, 0.01)) for c in ("Hx", "Hy", "Hz")})
        out.append(SimpleNamespace(mode_number=k, neff=2.4 - 0.1 * k, frequency=193e12 + 5e12 * k,
                                   wavelength=299792458.0 / (193e12 + 5e12 * k), x=u, y=v, power=1.0, **f))
    return out
