"""CPU oracle for the FDTD hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in NumPy float64, the reference Prismo time stepper
(``core/solver.py``), its grid semantics (``core/grid.py``), the CPML
coefficient formulas (``boundaries/pml.py``), the dispersive-material ADE
coefficients (``materials/dispersion.py``, ``materials/ade.py``), the soft
sources (``sources/*.py``) and the DFT running sum of ``monitors/field.py``.

It is the checker for the CUDA path and is imported only by ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py``.  Nothing in ``prismo_gb300`` imports it.

Two levels are provided:

* ``legacy=True`` (L0) reproduces the unmodified reference stepper exactly,
  including its H-update index offset and 2D sign flips.  It is pinned against
  fixtures produced by running the reference itself (``tests/golden``).
* ``legacy=False`` (L1) is the corrected stepper: the same coefficients,
  interpolation and curl expressions, with H written to ``H[..., 1:-1, ...]``
  (backward differences) and the 2D Ez-family H signs fixed, plus CPML,
  ADE coupling, soft sources, a 1D-auxiliary-grid TFSF plane and the DFT.
"""

from .fdtd64 import (  # noqa: F401
    C0,
    EPS0,
    MU0,
    COMPONENTS,
    OracleGrid,
    OracleFDTD,
    cpml_profile,
    lorentz_coeffs,
    drude_coeffs,
    debye_coeffs,
    gaussian_pulse,
    continuous_wave,
)
