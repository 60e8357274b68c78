"""CPU checks of the C ABI: the library builds, loads and exports every symbol
that include/prismo_cuda.h declares (no compute calls: there is no GPU here)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            src = open(os.path.join(ROOT, "include", f)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(pc_\w+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    from prismo_gb300 import _lib, build

    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def test_header_declares_api():
    names = declared_symbols()
    assert {"pc_create", "pc_step", "pc_destroy", "pc_set_fields", "pc_status"} <= names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_bindings_cover_header(lib):
    from prismo_gb300 import _lib

    assert declared_symbols() == set(_lib.SIGNATURES)


def test_version_and_invalid_args_without_gpu(lib):
    assert lib.pc_version() >= 100
    from prismo_gb300 import _lib

    d = _lib.GridDesc()
    d.ndim = 4  # invalid -> rejected before any CUDA call
    out = ctypes.c_void_p()
    assert lib.pc_create(ctypes.byref(d), ctypes.byref(out)) == _lib.PC_ERR_INVALID
    assert lib.pc_cpml_psi_elems(ctypes.byref(d), 4) == 0
    d.ndim, d.nx, d.ny, d.nz, d.pitch, d.precision = 3, 16, 16, 16, 32, 4
    d.mode, d.sched, d.dt, d.dx, d.dy, d.dz = 0, 0, 1e-17, 2e-8, 2e-8, 2e-8
    # two slabs of 3 per axis, four slots per axis
    want = 4 * (6 * 16 * 32) + 4 * (16 * 6 * 32) + 4 * (16 * 16 * 6)
    assert lib.pc_cpml_psi_elems(ctypes.byref(d), 3) == want
    d.pitch = 20  # not a multiple of 32
    assert lib.pc_cpml_psi_elems(ctypes.byref(d), 3) == 0


def test_error_mapping():
    from prismo_gb300 import _lib

    with pytest.raises(ValueError):
        _lib.check(_lib.PC_ERR_INVALID, "x")
    with pytest.raises(TimeoutError):
        _lib.check(_lib.PC_ERR_TIMEOUT, "x")
    with pytest.raises(FloatingPointError):
        _lib.check(_lib.PC_ERR_NONFINITE, "x")
    assert _lib.check(3) == 3


def test_batch_create_rejects_bad_instances_without_gpu(lib):
    """Instance validation happens before any CUDA call."""
    from prismo_gb300 import _lib

    inst = (_lib.BatchInstance * 1)()
    inst[0].nx, inst[0].ny = 30, 30  # too small for a 20-cell CPML
    inst[0].src_x, inst[0].src_y0, inst[0].src_n = 5, 5, 4
    h = ctypes.c_void_p()
    lay = _lib.BatchLayout()
    assert lib.pc_batch_create(1, inst, 20, 2e-8, 2e-8, 1e-17, 1e-11, ctypes.byref(h), ctypes.byref(lay)) \
        == _lib.PC_ERR_INVALID
    inst[0].nx, inst[0].ny = 100, 100
    inst[0].nport = 1
    inst[0].port_x[0], inst[0].port_y0[0], inst[0].port_n[0] = 50, 95, 10  # runs past the Ez extent
    assert lib.pc_batch_create(1, inst, 20, 2e-8, 2e-8, 1e-17, 1e-11, ctypes.byref(h), ctypes.byref(lay)) \
        == _lib.PC_ERR_INVALID
    assert lib.pc_batch_num_variants() >= 4
    out = (ctypes.c_int32 * 3)()
    assert lib.pc_batch_variant_info(0, out) == 0 and out[2] == 1
    assert lib.pc_batch_variant_info(99, out) == _lib.PC_ERR_INVALID


def test_monitor_port_tensor_entry_points_reject_bad_args_without_gpu(lib):
    """The plane-monitor, mode-port and anisotropic entry points validate their
    arguments before any CUDA call."""
    from prismo_gb300 import _lib

    INV = _lib.PC_ERR_INVALID
    comps = (ctypes.c_int32 * 4)(1, 5, 2, 4)
    offs = (ctypes.c_int64 * 4)(0, 0, 0, 0)
    w = (ctypes.c_double * 8)()
    n = ctypes.c_int64(0)
    assert lib.pc_add_flux(None, comps, offs, 1, 1.0, None, 16) == INV
    assert lib.pc_flux_count(None, 0, ctypes.byref(n), None) == INV
    assert lib.pc_flux_spectrum(None, comps, 1.0, None, None) == INV
    assert lib.pc_add_mode_monitor(None, comps, offs, 1, 1, w, None, 16) == INV
    assert lib.pc_mode_count(None, 0, ctypes.byref(n), None) == INV
    assert lib.pc_mode_spectrum(None, 0, w, 1, 0.0, 1e-17, None, None) == INV
    P3 = ctypes.c_void_p * 3
    nul = P3(None, None, None)
    assert lib.pc_aniso_update(2, 1, 1, nul, nul, nul, 4, None, w, 1.0, None) == INV  # precision
    assert lib.pc_aniso_update(4, 1, 0, nul, nul, nul, 4, None, w, 1.0, None) == INV  # sign
    assert lib.pc_aniso_update(4, 1, 1, nul, nul, nul, 4, None, None, 1.0, None) == INV  # no coefficients
    assert lib.pc_aniso_update(4, 1, 1, nul, nul, nul, 4, None, w, 1.0, None) == INV  # null arrays
    assert lib.pc_scatter_add(4, None, None, None, 4, 1.0, None) == INV
    assert lib.pc_scatter_add(3, None, None, None, 0, 1.0, None) == INV
    P4 = ctypes.c_void_p * 4
    assert lib.pc_plane_overlap(4, P4(None, None, None, None), None, 1, 1, None, None, None) == INV
    assert lib.pc_plane_overlap(8, None, None, 0, 1, None, None, None) == INV
