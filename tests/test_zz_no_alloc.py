"""The allocation-free entry point (pc_fused_steps_noalloc) against the
context-based one, through the C ABI.

It exists for callers that may not allocate device memory (a host application
whose device memory belongs to its own pool allocator, or a time loop that must
not take cudaMalloc's latency and synchronisation); its scratch is a fixed array
inside the library.  This file is collected last so that a run stopping at the
first failure has already run every other test.
"""

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(torch, precision, seed=17):
    from oracle import fdtd64 as O
    from prismo_gb300 import _lib
    from prismo_gb300.engine import COMPONENTS, FDTDEngine

    g = O.OracleGrid.from_total(70, 66, 100, 20e-9, 3)
    dt = g.suggest_dt(0.5)
    rng = np.random.default_rng(seed)
    eps = rng.uniform(1.0, 12.0, size=g.dims)
    init = {c: rng.standard_normal(g.shape(c)) * (1.0 if c[0] == "E" else 1 / 377.0) for c in COMPONENTS}

    eng = FDTDEngine(g.dims, g.spacing, dt, is_2d=False, precision=precision, sched="fused",
                     material_arrays={"eps_rel": eps})
    for c in COMPONENTS:
        eng.component(c).copy_(torch.from_numpy(init[c]).to(eng.device, eng.dtype))

    # caller-owned buffers for the allocation-free call: two field sets, Cb from the engine
    sets = [torch.zeros_like(eng.sets[0]), torch.zeros_like(eng.sets[0])]
    sets[0].copy_(eng.sets[eng.cur])
    lib = _lib.load()
    s0 = _lib.P6(*[sets[0][q].data_ptr() for q in range(6)])
    s1 = _lib.P6(*[sets[1][q].data_ptr() for q in range(6)])
    cb = _lib.P3(*[eng.coef[q].data_ptr() for q in range(3)])
    stream = torch.cuda.current_stream().cuda_stream
    return lib, eng, sets, s0, s1, cb, stream


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_no_alloc_steps_match_context_steps_twice(precision):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from prismo_gb300.engine import COMPONENTS

    lib, eng, sets, s0, s1, cb, stream = _setup(torch, precision)
    tol = 1e-5 if precision == "fp32" else 1e-12
    cur = 0
    for call in range(2):  # two calls in a row, each continuing from the last
        n = 9 + call
        eng.step(n)
        st = C.c_uint32(7)
        cur = lib.pc_fused_steps_noalloc(C.byref(eng.desc), s0, s1, cur, cb, n, stream, C.byref(st))
        assert cur in (0, 1), cur
        assert st.value == 0
        torch.cuda.synchronize()
        for c in COMPONENTS:
            want = eng.component(c).double().cpu().numpy()
            shp = want.shape
            got = sets[cur][COMPONENTS.index(c)][: shp[0], : shp[1], : shp[2]].double().cpu().numpy()
            err = np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300)
            assert err <= tol, (call, c, err)
    eng.close()


def test_no_alloc_calls_leave_device_memory_unchanged():
    """After a first call (which resolves the scratch address), further calls
    take no device memory: the free-memory figure stays the same."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib, eng, sets, s0, s1, cb, stream = _setup(torch, "fp32", seed=3)
    cur = lib.pc_fused_steps_noalloc(C.byref(eng.desc), s0, s1, 0, cb, 2, stream, None)
    assert cur in (0, 1)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        st = C.c_uint32(0)
        cur = lib.pc_fused_steps_noalloc(C.byref(eng.desc), s0, s1, cur, cb, 3, stream, C.byref(st))
        assert cur in (0, 1) and st.value == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    eng.close()


def test_no_alloc_reports_nonfinite_fields():
    """A NaN written into the input fields from the host comes back as the
    non-finite status bit; the next clean call resets the word."""
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from prismo_gb300 import _lib

    lib, eng, sets, s0, s1, cb, stream = _setup(torch, "fp32", seed=5)
    sets[0][1][30, 31, 40] = float("nan")  # Ey, inside the grid
    st = C.c_uint32(0)
    cur = lib.pc_fused_steps_noalloc(C.byref(eng.desc), s0, s1, 0, cb, 2, stream, C.byref(st))
    assert cur in (0, 1)
    assert st.value & _lib.PC_STATUS_NONFINITE, st.value
    for q in range(2):
        sets[q].zero_()
    cur = lib.pc_fused_steps_noalloc(C.byref(eng.desc), s0, s1, 0, cb, 2, stream, C.byref(st))
    assert cur in (0, 1) and st.value == 0, st.value
    eng.close()


def test_no_alloc_rejects_oversized_and_invalid():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from prismo_gb300 import _lib

    lib = _lib.load()
    d = _lib.GridDesc()
    d.ndim, d.nx, d.ny, d.nz, d.pitch, d.precision = 2, 16, 16, 1, 32, 4  # 2D: not supported
    d.mode, d.sched, d.dt, d.dx, d.dy, d.dz = 0, 0, 1e-17, 2e-8, 2e-8, 0.0
    z = _lib.P6(*([1] * 6))
    cb = _lib.P3(*([1] * 3))
    assert lib.pc_fused_steps_noalloc(C.byref(d), z, z, 0, cb, 1, None, None) == _lib.PC_ERR_INVALID
    # more work items than the fixed scratch holds (256 x 512 tiles): rejected before any launch
    d.ndim, d.nx, d.ny, d.nz, d.pitch = 3, 16, 8192, 8192, 8192
    d.dz = 2e-8
    assert lib.pc_fused_steps_noalloc(C.byref(d), z, z, 0, cb, 1, None, None) == _lib.PC_ERR_INVALID
