"""ctypes binding of libprismo_cuda.so (the C ABI in include/prismo_cuda.h).

The library must be built (``prismo_gb300.build.build()``) and loadable; there is
no CPU fallback: every entry point raises if the native library is missing.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libprismo_cuda.so")

PC_OK = 0
PC_ERR_INVALID = -1
PC_ERR_CUDA = -2
PC_ERR_TIMEOUT = -3
PC_ERR_NONFINITE = -4
PC_ERR_STATE = -5

PC_STATUS_NONFINITE = 0x1
PC_STATUS_TIMEOUT = 0x2
PC_STATUS_BOUNDS = 0x4

PC_MODE_CORRECTED = 0
PC_MODE_LEGACY = 1

PC_SCHED_AUTO = 0
PC_SCHED_SPLIT = 1
PC_SCHED_FUSED = 2

PC_TUNE_FUSED_CHUNK = 1
PC_TUNE_FUSED_CHUNK_EDGE = 3
PC_TUNE_FUSED_SPLIT = 4
PC_TUNE_FUSED_UNIFIED = 5
PC_TUNE_GRAPH_STEPS = 2
PC_TUNE_TS_STEPS = 6
PC_TUNE_TS_CHUNK = 7
PC_TUNE_TS_ORDER = 8
PC_TUNE_TS_ACTIVE = 9
PC_TUNE_FUSED_EXTRAS = 10


class GridDesc(C.Structure):
    _fields_ = [
        ("ndim", C.c_int32),
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("nz", C.c_int32),
        ("pitch", C.c_int32),
        ("precision", C.c_int32),
        ("mode", C.c_int32),
        ("sched", C.c_int32),
        ("dt", C.c_double),
        ("dx", C.c_double),
        ("dy", C.c_double),
        ("dz", C.c_double),
    ]


class AdeRegion(C.Structure):
    _fields_ = [
        ("box", C.c_int32 * 6),
        ("npoles", C.c_int32),
        ("kind", C.c_int32 * 4),
        ("eps_inf", C.c_double),
        ("c0", C.c_double * 4),
        ("c1", C.c_double * 4),
        ("c2", C.c_double * 4),
        ("c3", C.c_double * 4),
        ("aux", ((C.c_void_p * 2) * 4) * 3),
    ]


P6 = C.c_void_p * 6
P3 = C.c_void_p * 3
D3 = C.POINTER(C.c_double) * 3
VPP = C.POINTER(C.c_void_p)  # void* const x[n]
DPP = C.POINTER(C.POINTER(C.c_double))  # const double* const x[3]

# name -> (restype, argtypes); every symbol declared in include/prismo_cuda.h
class BatchInstance(C.Structure):
    _fields_ = [
        ("nx", C.c_int32),
        ("ny", C.c_int32),
        ("src_x", C.c_int32),
        ("src_y0", C.c_int32),
        ("src_n", C.c_int32),
        ("nport", C.c_int32),
        ("port_x", C.c_int32 * 4),
        ("port_y0", C.c_int32 * 4),
        ("port_n", C.c_int32 * 4),
    ]


class BatchLayout(C.Structure):
    _fields_ = [
        ("field_elems", C.c_int64),
        ("coef_elems", C.c_int64),
        ("psi_elems", C.c_int64),
        ("weight_elems", C.c_int64),
        ("dft_points", C.c_int64),
    ]


SIGNATURES = {
    "pc_version": (C.c_int, []),
    "pc_create": (C.c_int, [C.POINTER(GridDesc), C.POINTER(C.c_void_p)]),
    "pc_destroy": (None, [C.c_void_p]),
    "pc_set_fields": (C.c_int, [C.c_void_p, VPP, VPP]),
    "pc_current_set": (C.c_int, [C.c_void_p]),
    "pc_set_current_set": (C.c_int, [C.c_void_p, C.c_int32]),
    "pc_build_coefficients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double,
                                        C.c_double, VPP, VPP, VPP, VPP, C.c_void_p]),
    "pc_set_coefficients": (C.c_int, [C.c_void_p, VPP, VPP, VPP, VPP, C.c_double, C.c_double]),
    "pc_cpml_psi_elems": (C.c_size_t, [C.POINTER(GridDesc), C.c_int32]),
    "pc_set_cpml": (C.c_int, [C.c_void_p, C.c_int32, DPP, DPP, DPP, C.c_void_p, C.c_void_p]),
    "pc_add_source": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.c_int32]),
    "pc_step": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_void_p]),
    "pc_set_tfsf": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_double,
                              C.c_double]),
    "pc_set_ade": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(AdeRegion), C.c_double]),
    "pc_add_dft": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.c_int32, C.POINTER(C.c_double),
                             C.c_int32, C.c_double, C.c_double, C.c_void_p]),
    "pc_dft_flush": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "pc_add_flux": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.c_int32, C.c_double,
                              C.c_void_p, C.c_int64]),
    "pc_flux_count": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.c_void_p]),
    "pc_flux_spectrum": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_double, C.c_void_p, C.c_void_p]),
    "pc_aniso_update": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                  C.POINTER(C.c_void_p), C.c_int64, C.c_void_p, C.POINTER(C.c_double), C.c_double,
                                  C.c_void_p]),
    "pc_scatter_add": (C.c_int, [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_double,
                                 C.c_void_p]),
    "pc_plane_overlap": (C.c_int, [C.c_int32, C.POINTER(C.c_void_p), C.c_void_p, C.c_int32, C.c_int32, C.c_void_p,
                                   C.c_void_p, C.c_void_p]),
    "pc_add_mode_monitor": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.c_int32, C.c_int32,
                                      C.POINTER(C.c_double), C.c_void_p, C.c_int64]),
    "pc_mode_count": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64), C.c_void_p]),
    "pc_mode_spectrum": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_double), C.c_int32, C.c_double, C.c_double,
                                   C.c_void_p, C.c_void_p]),
    "pc_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p]),
    "pc_launch_count": (C.c_int64, [C.c_void_p]),
    "pc_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int64]),
    "pc_get_tuning": (C.c_int64, [C.c_void_p, C.c_int32]),
    "pc_fused_steps_noalloc": (C.c_int, [C.POINTER(GridDesc), VPP, VPP, C.c_int32, VPP, C.c_int32, C.c_void_p,
                                         C.POINTER(C.c_uint32)]),
    "pc_profile": (C.c_int, [C.c_void_p, C.c_int32]),
    "pc_profile_read": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    "pc_profile_steps": (C.c_int64, [C.c_void_p]),
    "pc_batch_create": (C.c_int, [C.c_int32, C.POINTER(BatchInstance), C.c_int32, C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.POINTER(C.c_void_p), C.POINTER(BatchLayout)]),
    "pc_batch_instance_offsets": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "pc_batch_bind": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "pc_batch_build_coefficients": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_double, C.c_void_p]),
    "pc_batch_set_cpml": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]),
    "pc_batch_set_sources": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int32]),
    "pc_batch_set_dft": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_int32, C.c_double, C.c_void_p]),
    "pc_batch_num_variants": (C.c_int, []),
    "pc_batch_variant_info": (C.c_int, [C.c_int32, C.POINTER(C.c_int32)]),
    "pc_batch_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "pc_batch_get_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]),
    "pc_batch_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.c_void_p]),
    "pc_batch_step": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "pc_batch_dft_flush": (C.c_int, [C.c_void_p, C.c_void_p]),
    "pc_batch_current_set": (C.c_int, [C.c_void_p]),
    "pc_batch_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p]),
    "pc_batch_instance_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p]),
    "pc_batch_launch_count": (C.c_int64, [C.c_void_p]),
    "pc_batch_steps_done": (C.c_int64, [C.c_void_p]),
    "pc_batch_destroy": (None, [C.c_void_p]),
    "pc_mlp_create": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_void_p)]),
    "pc_mlp_param_count": (C.c_int64, [C.c_void_p]),
    "pc_mlp_param_layout": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int64)]),
    "pc_mlp_set_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "pc_mlp_get_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "pc_mlp_get_grads": (C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    "pc_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "pc_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "pc_mlp_train_step": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_float,
                                    C.c_float, C.c_void_p, C.c_void_p]),
    "pc_mlp_launch_count": (C.c_int64, [C.c_void_p]),
    "pc_mlp_set_tensor_path": (C.c_int, [C.c_void_p, C.c_int32]),
    "pc_mlp_status": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint32), C.c_void_p]),
    "pc_mlp_destroy": (None, [C.c_void_p]),
}

_lock = threading.Lock()
_lib = None


class NativeLibraryMissing(RuntimeError):
    pass


def load():
    """Load (once) and return the native library; raise if it is absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise NativeLibraryMissing(
                f"{LIB_PATH} is not built; run prismo_gb300.build.build() (nvcc, sm_103a)")
        lib = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int, what: str = "") -> int:
    """Map a negative PC_ERR_* code to a Python exception."""
    if rc >= 0:
        return rc
    msg = f"{what} failed with code {rc}"
    if rc == PC_ERR_INVALID:
        raise ValueError(msg + " (invalid argument)")
    if rc == PC_ERR_TIMEOUT:
        raise TimeoutError(msg)
    if rc == PC_ERR_NONFINITE:
        raise FloatingPointError(msg)
    if rc == PC_ERR_STATE:
        raise RuntimeError(msg + " (call out of order)")
    raise RuntimeError(msg + " (CUDA error)")


def ptr3(ts):
    """ctypes array of three device pointers (None -> NULL) from tensors."""
    arr = P3()
    for i, t in enumerate(ts):
        arr[i] = None if t is None else t.data_ptr()
    return arr
