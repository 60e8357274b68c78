"""Benchmark: 3D FP32 CPML FDTD, 256^3 cells, 2000 time steps (one "step" of this
benchmark = one whole 2000-time-step simulation from zero fields).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--chunk CX[,EDGE]]
    python bench.py --workload 2d|dispersive|sweep|surrogate   (the other configurations)
    python bench.py --workload mlp                             (the surrogate's products, forward and training)

Workload (the reference's 3D plain-FDTD configuration): 256^3 total cells at
dx = 20 nm with a 12-cell CPML on all six faces, Courant 0.5, 32 seeded
dielectric boxes (eps in [1, 12.11]) on eps = 2.085, an Ez point dipole at the
centre driven by a 193 THz / 10 fs Gaussian pulse, 2000 steps.  Metric:
Gcell-updates/s (one cell advanced one full step = one update).

Prints one JSON line (rank 0).  Multi-GPU runs are independent replicas (the
single-grid stepper does not shard); value = all ranks' updates / max time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DIMS = (256, 256, 256)
DX = 20e-9
CPML = 12
TSTEPS = 2000
COURANT = 0.5
# algorithmic bytes per cell-update of the fused stepper, float32:
#   6 fields read + written (48 B) + Cb for Ex, Ey, Ez read (12 B) = 60 B,
#   plus the CPML psi recursions: 4 psi arrays read + written (32 B) on the
#   slab cells, 3 axes x 2 x 12 / 256 of the cells -> 9.0 B on average.
B_INTERIOR = 60.0
B_CPML_PER_SLAB_CELL = 32.0


def b_alg(dims=DIMS, t=CPML):
    frac = sum(2.0 * t / n for n in dims)
    return B_INTERIOR + B_CPML_PER_SLAB_CELL * frac


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_value(name, dims, key):
    """A figure from a committed ncu summary (profiles/<name>) for the grid it covers."""
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if tuple(d.get("dims", ())) == tuple(dims):
            return d.get(key)
    return None


def traffic_from_profile(dims, name="fused3_256_cpml.json"):
    """DRAM bytes per launch of the stencil kernel from a committed ncu summary
    (None for a grid the summary does not cover)."""
    p = os.path.join(ROOT, "profiles", name)
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        if tuple(d.get("dims", ())) == tuple(dims):
            return d.get("dram_bytes_per_launch")
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return out
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in rows:
            for name, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        out["sm_mhz"] = statistics.median(loaded) if loaded else None
        out["sm_max_mhz"] = max(mx) if mx else None
        out["reasons"] = sorted(reasons)
        out["samples"] = len(rows)
        return out


def make_engine(eps, precision="fp32", dims=DIMS):
    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.grid import YeeGrid
    from prismo_gb300.pml import PMLParams
    from prismo_gb300.sources import GaussianPulse

    grid = YeeGrid.from_total(dims, DX, CPML)
    dt = grid.suggest_time_step(COURANT)
    eng = FDTDEngine(grid.dimensions, grid.spacing, dt, is_2d=False, precision=precision,
                     material_arrays={"eps_rel": eps}, pml=PMLParams(thickness=CPML))
    wf = GaussianPulse(193e12, 10e-15)
    c = tuple(n // 2 for n in dims)
    idx = (np.array([c[0]]).reshape(1, 1, 1), np.array([c[1]]).reshape(1, 1, 1), np.array([c[2]]).reshape(1, 1, 1))
    eng.add_source("Ez", eng.offsets("Ez", idx), None, wf)
    times = np.cumsum(np.full(TSTEPS, dt))
    amps = np.asarray(wf(times), dtype=np.float64).reshape(TSTEPS, 1)
    return grid, eng, amps


def reset(eng):
    for s in eng.sets:
        s.zero_()
    for p in eng.psi:
        p.zero_()
    eng.lib.pc_set_current_set(eng.ctx, 0)


def cpu_baseline_sample(dims=DIMS, nsteps=3):
    """FP64 oracle stepper (corrected, CPML) on this host: a bounded sample."""
    from oracle import fdtd64 as O
    from prismo_gb300.workloads import boxes_3d

    g = O.OracleGrid.from_total(*dims, DX, CPML)
    dt = g.suggest_dt(COURANT)
    eps = boxes_3d(dims, seed=0)
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=CPML)
    o.F["Ez"][dims[0] // 2, dims[1] // 2, dims[2] // 2] = 1.0
    o.step()  # warm-up (allocates psi)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        o.step()
    el = time.perf_counter() - t0
    cells = dims[0] * dims[1] * dims[2]
    return cells * nsteps / el / 1e9, el


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_throughput(ms_local: float, units_per_rank: float, device=None):
    """(max over ranks of the timed milliseconds, whole-job units per second).
    The job ends when its slowest replica does, and every rank processed
    ``units_per_rank``; a single process reports its own time."""
    import torch

    ws = dist_env()[0]
    ms = float(ms_local)
    if ws > 1 and torch.distributed.is_available() and torch.distributed.is_initialized():
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, units_per_rank * ws / (ms / 1e3)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import fdtd64 as O
    from prismo_gb300.workloads import boxes_3d

    dims = DIMS
    g = O.OracleGrid.from_total(*dims, DX, CPML)
    dt = g.suggest_dt(COURANT)
    eps = boxes_3d(dims, seed=0)
    o = O.OracleFDTD(g, dt, {"eps_rel": eps}, cpml_layers=CPML)
    wf = O.gaussian_pulse(193e12, 10e-15)
    c = tuple(n // 2 for n in dims)
    o.add_source("Ez", (np.array([[[c[0]]]]), np.array([[[c[1]]]]), np.array([[[c[2]]]])), wf)
    per = 1  # time steps per bench step: a bounded sample of the 2000-step run
    for _ in range(args.warmup):
        o.run(per)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.run(per)
    el = time.perf_counter() - t0
    cells = float(np.prod(dims))
    value = cells * per * args.steps / el / 1e9
    # the unmodified reference stepper (MaxwellUpdater.step, core/solver.py:535-552,
    # imported from the installed copy under baseline/_ref): no CPML, and unstable,
    # so only its time per step on the same grid is reported
    l0 = reference_l0_timing(dims, eps, dt)
    line = {
        "impl": "reference", "metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "3d_fp32_cpml_256: 256^3, dx=20nm, 12-cell CPML, 32 seeded boxes, Ez dipole, 2000 steps",
                   "sample": f"{per} time step(s) of the 2000 per bench step", "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": value, "unit": "Gcell/s", "cores": 1, "kind": "port",
                         "sample": f"{per} of 2000 time steps per bench step, NumPy float64 oracle, 1 thread"},
        "e2e": {"value": value, "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_stepper_l0": l0,
    }
    print(json.dumps(line), flush=True)


def reference_l0_timing(dims, eps, dt, steps=2):
    """Time per step of the unmodified reference MaxwellUpdater on this grid (the
    reference package installed under baseline/_ref), or why it could not run."""
    import builtins
    import types

    path = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(path, "prismo")):
        return {"unavailable": "reference package not installed under baseline/_ref"}
    try:
        builtins.MTLBuffer = object  # the reference's metal backend annotates with it unguarded
        pl = types.ModuleType("polars")
        pl.DataFrame = object
        sys.modules.setdefault("polars", pl)
        try:  # a dependency of the reference's sweep module only, absent on some machines
            import tqdm  # noqa: F401
        except ImportError:
            tq = types.ModuleType("tqdm")
            tq.tqdm = lambda it=None, *a, **k: it
            sys.modules["tqdm"] = tq
        if path not in sys.path:
            sys.path.insert(0, path)
        from prismo.core.fields import ElectromagneticFields
        from prismo.core.grid import GridSpec, YeeGrid
        from prismo.core.solver import MaxwellUpdater

        n = dims[0]
        size = tuple((d - 2 * CPML - 0.5) * DX for d in dims)
        grid = YeeGrid(GridSpec(size=size, resolution=1.0 / DX, boundary_layers=CPML))
        upd = MaxwellUpdater(grid, dt, material_arrays={"eps_rel": eps})
        fields = ElectromagneticFields(grid)
        upd.step(fields)
        t0 = time.perf_counter()
        for _ in range(steps):
            upd.step(fields)
        el = (time.perf_counter() - t0) / steps
        return {"value": float(np.prod(grid.dimensions)) / el / 1e9, "unit": "Gcell/s", "ms_per_step": el * 1e3,
                "cores": 1, "grid": list(grid.dimensions), "steps_timed": steps,
                "api": "prismo.core.solver.MaxwellUpdater.step (unmodified; no CPML)", "n": n}
    except Exception as e:  # noqa: BLE001 - report, never fail the bench line
        return {"unavailable": f"{type(e).__name__}: {e}"[:200]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--tsteps", type=int, default=TSTEPS, help="time steps per bench step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--chunk", default=None,
                    help="x-chunk lengths 'CX[,EDGE]' of the fused schedule instead of autotuning (profiling runs)")
    ap.add_argument("--time-blocking", type=int, default=2, choices=[0, 1, 2],
                    help="time steps per launch of the temporally blocked stepper (0: the one-step fused schedule)")
    ap.add_argument("--ts-chunk", type=int, default=0, help="x-chunk of the temporally blocked stepper (0: auto)")
    ap.add_argument("--dims", type=int, default=None,
                    help="cube edge for a reduced profiling case (default: the 256^3 workload)")
    ap.add_argument("--workload", default="3d", choices=["3d", "2d", "dispersive", "sweep", "surrogate", "mlp"],
                    help="3d: the headline 256^3 CPML workload; dispersive: 384x384x192 Drude-Lorentz + TFSF + "
                         "64-frequency DFT planes; sweep: 64 batched couplers; surrogate: train + held-out pipeline; "
                         "mlp: the surrogate's forward products alone (tcgen05 and mma.sync)")
    ap.add_argument("--designs", type=int, default=64, help="designs per batched sweep")
    ap.add_argument("--dispersive-schedule", default="fused", choices=["fused", "split"],
                    help="dispersive workload: fused H + E kernel with the ADE pole pass, or the split kernels")
    args = ap.parse_args()
    if args.workload != "3d":
        return run_other(args)
    global DIMS
    if args.dims:
        DIMS = (args.dims,) * 3
    if args.impl == "reference":
        run_reference(args)
        return
    import torch

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device(f"cuda:{local}")
    torch.cuda.set_device(dev)

    from prismo_gb300.workloads import boxes_3d

    eps = boxes_3d(DIMS, seed=0)
    grid, eng, amps_full = make_engine(eps, dims=DIMS)
    tsteps = args.tsteps
    amps = amps_full[:tsteps]
    cells = float(np.prod(DIMS))
    stream = eng.stream

    def one():
        reset(eng)
        eng.step(tsteps, amps)

    eng.set_time_blocking(args.time_blocking, args.ts_chunk)
    if args.chunk:
        cx, _, ce = args.chunk.partition(",")
        eng.set_chunk(int(cx), int(ce or 0))
        tuned_chunk = (int(cx), int(ce or 0))
    else:
        tuned_chunk = None if args.no_autotune else eng.autotune(cache=False)
    for _ in range(max(args.warmup, 3)):
        one()
    eng.synchronize()
    status = eng.check_status()

    clocks = ClockSampler(local)
    clocks.start()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    n0 = eng.launch_count()
    eng.profile(True)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        one()
    ev1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ms_total = ev0.elapsed_time(ev1)
    kern_ms, kern_n, kern_steps = eng.profile_read()
    eng.profile(False)
    launches = eng.launch_count() - n0
    clk = clocks.stop()
    status |= eng.check_status()
    ms_total, units_per_s = replica_throughput(ms_total, cells * tsteps * args.steps, dev)
    value = units_per_s / 1e9

    # roofline of the dominant kernel: the temporally blocked stepper (one launch =
    # two time steps) or the fused H+E stencil (one launch = one time step).
    # achieved = the per-time-step algorithmic bytes (69 B/cell) x the cells and
    # time steps one launch advances / the launch time: with two steps per launch
    # it can exceed the copy bandwidth, which is what the blocking is for.
    blocked = eng.time_blocking_active() and args.time_blocking > 0
    bpc = b_alg(DIMS)
    avg_launch_s = kern_ms / 1e3 / max(kern_n, 1)
    steps_per_launch = kern_steps / max(kern_n, 1)
    achieved = bpc * cells * steps_per_launch / avg_launch_s / 1e9  # GB/s
    peak, peak_kind = measured_peaks()
    traffic = traffic_from_profile(DIMS, "ts3_256_cpml.json" if blocked else "fused3_256_cpml.json")

    # end-to-end through the engine API with host buffers
    e2e = None
    if not args.no_e2e and rank == 0:
        e2e = run_e2e(eng, eps, amps, tsteps, cells)

    cpu = None
    if not args.no_cpu_baseline and rank == 0:
        v, el = cpu_baseline_sample(dims=DIMS, nsteps=3)
        cpu = {"value": v, "unit": "Gcell/s", "cores": 1, "kind": "port",
               "sample": f"3 time steps (of 2000) of the 256^3 CPML stepper, NumPy float64 oracle, {el:.1f} s"}

    if rank == 0:
        line = {
            "metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "3d_fp32_cpml_256: 256^3 total cells, dx=20nm, 12-cell CPML, Courant 0.5, "
                                   "32 seeded boxes eps U[1,12.11] on 2.085, Ez dipole 193THz/10fs",
                       "time_steps_per_step": tsteps, "parallelism": "replicas" if ws > 1 else "single",
                       "l2": "inputs larger than L2 (fields 2x403 MB)", "status": status,
                       "schedule": "temporally blocked, 2 time steps per launch" if blocked else "fused, 1 step per launch",
                       "tuned": None if tuned_chunk is None else list(tuned_chunk)},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "bytes_per_cell_update": bpc,
                         "kernel": "ts3_multi<2> (H+E+CPML, 2 steps)" if blocked else "fused3 (H+E+CPML)",
                         "time_steps_per_launch": steps_per_launch,
                         "compulsory_frac": bpc * cells / avg_launch_s / 1e9 / peak,
                         "avg_launch_us": avg_launch_s * 1e6, "launches_timed": kern_n},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    eng.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def run_e2e(eng, eps, amps, tsteps, cells, reps=2):
    """Host inputs -> device -> simulate -> host outputs, per step."""
    import torch

    eps_h = torch.from_numpy(eps).pin_memory()
    outs = [torch.empty(tuple(eng.component(c).shape), dtype=eng.dtype).pin_memory()
            for c in ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")]
    stream = eng.stream
    h2d = eps_h.numel() * eps_h.element_size()
    d2h = sum(o.numel() * o.element_size() for o in outs)

    def one():
        eps_d = eps_h.to(eng.device, non_blocking=True)
        eng._set_materials({"eps_rel": eps_d})
        reset(eng)
        eng.step(tsteps, amps)
        for o, c in zip(outs, ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")):
            o.copy_(eng.component(c), non_blocking=True)

    one()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(reps):
        one()
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    return {"value": cells * tsteps / (ms / 1e3) / 1e9, "unit": "Gcell/s", "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": ms, "api": "prismo_gb300.engine.FDTDEngine (host eps in, host fields out)"}


# ---------------------------------------------------------------------------
# the other configurations (run by hand: python bench.py --workload ...)
# ---------------------------------------------------------------------------
def _line(**kw):
    base = {"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic"}
    base.update(kw)
    print(json.dumps(base), flush=True)


def _oracle_coupler_worker(seed, nsteps):
    """One design's coupler + normalisation run on the float64 oracle, nsteps of
    the 4000 (a bounded sample); returns seconds per 4000-step design."""
    from oracle import fdtd64 as O
    from prismo_gb300 import sweep as S

    L = S.coupler_layout(S.coupler_design(seed))
    el = 0.0
    for eps, ports in ((L.eps, L.ports), (L.norm_eps, L.ports[:1])):
        nx, ny = eps.shape
        g = O.OracleGrid.from_total(nx, ny, 1, S.DX, S.CPML)
        o = O.OracleFDTD(g, S.sweep_dt(), {"eps_rel": eps[:, :, None]}, cpml_layers=S.CPML)
        o.add_source("Ez", (np.array([[L.src.x]]), np.arange(L.src.y0, L.src.y0 + L.src.n)[None, :]),
                     O.gaussian_pulse(S.F0, S.PULSE_WIDTH), weight=L.src.profile[None, :])
        for p in ports:
            o.add_dft("Ez", (np.array([[p.x]]), np.arange(p.y0, p.y0 + p.n)[None, :]), S.sweep_freqs(S.NFREQ))
        o.step()
        t0 = time.perf_counter()
        for _ in range(nsteps):
            o.step()
        el += (time.perf_counter() - t0) / nsteps * S.STEPS
    return el


def sweep_cpu_baseline(nsteps=10):
    """ParameterSweep(parallel=True) shape: one float64 oracle design per host core."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(cores) as pool:
        secs = pool.starmap(_oracle_coupler_worker, [(s, nsteps) for s in range(cores)])
    return sum(1.0 / x for x in secs), cores, float(np.mean(secs))


def run_other(args):
    if args.workload == "sweep" or args.workload == "surrogate":
        cpu = None
        if not args.no_cpu_baseline:  # before any GPU work: the pool is spawned
            v, cores, sec = sweep_cpu_baseline()
            cpu = {"value": v, "unit": "designs/s", "cores": cores, "kind": "port",
                   "sample": f"10 of 4000 steps of one coupler + normalisation per core, float64 oracle "
                             f"(ParameterSweep parallel shape), {sec:.0f} s per design extrapolated"}
    import torch

    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    peak, peak_kind = measured_peaks()
    if args.workload == "dispersive":
        return run_dispersive(args, peak, peak_kind)
    if args.workload == "2d":
        return run_2d(args)
    if args.workload == "sweep":
        return run_sweep(args, cpu, peak, peak_kind)
    if args.workload == "mlp":
        return run_mlp(args)
    return run_surrogate(args, cpu)


def run_2d(args):
    """The 2D TE drop-in configuration: 500 x 250 total cells, 20-cell CPML, slab
    waveguide, soft Ez line source, 11-frequency DFT line, 3000 steps (one bench
    step = the whole run from zero fields).  The grid (3 MB) lives in L2: the
    metric is steps/s and Gcell/s, not an HBM roofline."""
    import torch

    from prismo_gb300.engine import FDTDEngine
    from prismo_gb300.grid import YeeGrid
    from prismo_gb300.pml import PMLParams
    from prismo_gb300.sources import GaussianPulse
    from prismo_gb300.workloads import CONFIG_2D, config_2d_layout

    cfg = CONFIG_2D
    g = YeeGrid.from_total(cfg["dims"], cfg["dx"], cfg["cpml"])
    dt = g.suggest_time_step(cfg["courant"])
    eps, src, mon, freqs = config_2d_layout()
    n = cfg["steps"]
    wf = GaussianPulse(cfg["pulse_f0"], cfg["pulse_width"])
    amps = np.asarray(wf(np.cumsum(np.full(n, dt))), dtype=np.float64)[:, None]
    eng = FDTDEngine(g.dimensions, g.spacing, dt, is_2d=True, precision="fp32", material_arrays={"eps_rel": eps},
                     pml=PMLParams(thickness=cfg["cpml"]))
    eng.add_source("Ez", eng.offsets("Ez", src), None, wf)
    eng.add_dft("Ez", eng.offsets("Ez", mon), freqs, t0=dt)

    def one():
        for s_ in eng.sets:
            s_.zero_()
        for p_ in eng.psi:
            p_.zero_()
        eng.step(n, amps)

    for _ in range(max(args.warmup, 3)):
        one()
    eng.synchronize()
    n0 = eng.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(0)
    clocks.start()
    ev0.record(eng.stream)
    for _ in range(args.steps):
        one()
    ev1.record(eng.stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1) / args.steps
    cells = float(np.prod(g.dimensions))
    # CPU baseline: the float64 oracle, 50 steps of the same grid, 1 thread
    from oracle import fdtd64 as O

    go = O.OracleGrid.from_total(*cfg["dims"], cfg["dx"], cfg["cpml"])
    o = O.OracleFDTD(go, dt, {"eps_rel": eps}, cpml_layers=cfg["cpml"])
    o.add_source("Ez", src, O.gaussian_pulse(cfg["pulse_f0"], cfg["pulse_width"]))
    o.add_dft("Ez", mon, freqs)
    o.run(2)
    t0 = time.perf_counter()
    o.run(50)
    cpu_s = (time.perf_counter() - t0) / 50
    # The same simulation as a one-instance batch (csrc/batch.cu: K steps per launch
    # in shared memory): a secondary figure beside the drop-in engine's.  Fields
    # after one run from zero are compared with the engine's; the timed run
    # continues the same instance (the work does not depend on the field values).
    one()
    eng.synchronize()
    from prismo_gb300 import sweep as S

    core = np.asarray(src[1]).ravel()
    line = np.asarray(mon[1]).ravel()
    inst = S.Instance(eps=np.ascontiguousarray(eps[:, :, 0] if eps.ndim == 3 else eps), src=S.Port(int(np.ravel(src[0])[0]), int(core[0]), int(core.size), np.ones(core.size)),
                      ports=[S.Port(int(np.ravel(mon[0])[0]), int(line[0]), int(line.size), np.ones(line.size))])
    B = S.BatchedFDTD2D([inst], freqs, dx=cfg["dx"], dt=dt, cpml=cfg["cpml"])
    B.set_amplitudes(amps[:, 0])
    B.step(n)
    ez_b = B.fields(0)[0].float()
    ez_e = eng.component("Ez").float()
    r, c = min(ez_b.shape[0], ez_e.shape[0]), min(ez_b.shape[1], ez_e.shape[1])
    batch_rel = float((ez_b[:r, :c] - ez_e[:r, :c]).norm() / ez_e[:r, :c].norm().clamp_min(1e-30))
    bev0, bev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    bev0.record(B.stream)
    B.step(n)
    bev1.record(B.stream)
    torch.cuda.synchronize()
    batch_ms = bev0.elapsed_time(bev1)
    batch_tile = S.BatchedFDTD2D.variants()[B.tuning()[0]]
    B.close()
    _line(metric="Gcell-updates/s", value=cells * n / (ms / 1e3) / 1e9, unit="Gcell/s", steps=args.steps,
          warmup=args.warmup, ms_per_step=ms, dtype="f32",
          config={"workload": "2d_te_waveguide_500x250: 20-cell CPML, slab waveguide, soft Ez line source, "
                              "11-frequency DFT line, 3000 steps (L2-resident grid)",
                  "time_steps_per_s": n / (ms / 1e3), "l2": "grid fits L2 (launch/latency bound)"},
          same_simulation_on_batch_engine={"gcell_per_s": cells * n / (batch_ms / 1e3) / 1e9,
                                           "time_steps_per_s": n / (batch_ms / 1e3), "tile_steps": batch_tile,
                                           "ez_rel_l2_vs_engine": batch_rel},
          cpu_baseline={"value": cells / cpu_s / 1e9, "unit": "Gcell/s", "cores": 1, "kind": "port",
                        "sample": f"50 of 3000 steps, float64 oracle, {cpu_s * 1e3:.1f} ms/step"},
          gpu_launches=eng.launch_count() - n0, clocks=clk)
    eng.close()


def run_dispersive(args, peak, peak_kind):
    """384x384x192 Drude + 2 Lorentz metal, ridge, TFSF, two 64-frequency DFT
    planes; each bench step continues the simulation by --tsteps (default 400)
    time steps (warm-up + timed steps stay within the 4000-step run)."""
    import torch

    from prismo_gb300.workloads import CONFIG_3D_DISPERSIVE, build_dispersive_engine, dispersive_bytes_per_cell

    dims = CONFIG_3D_DISPERSIVE["dims"]
    per = args.tsteps if args.tsteps != TSTEPS else 400
    eng, info = build_dispersive_engine(dims)
    fused = args.dispersive_schedule == "fused"
    eng.set_fused_extras(fused)
    tuned = None
    if fused and args.chunk:  # fixed x-chunks (profiling runs)
        cx, _, ce = args.chunk.partition(",")
        eng.set_chunk(int(cx), int(ce or 0))
        tuned = [int(cx), int(ce or 0)]
    elif fused and not args.no_autotune:
        tuned = eng.autotune(cache=False)
    total = (args.warmup + args.steps) * per
    amps = info["waveform"]((np.arange(total) + 1) * info["dt"])[:, None]
    pos = 0

    def one():
        nonlocal pos
        eng.step(per, amps[pos:pos + per])
        pos += per

    for _ in range(args.warmup):
        one()
    eng.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    n0 = eng.launch_count()
    eng.profile(True)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(eng.stream)
    for _ in range(args.steps):
        one()
    ev1.record(eng.stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    kern_ms, kern_n, _ = eng.profile_read()
    clk = clocks.stop()
    status = eng.check_status()
    cells = float(np.prod(dims))
    value = cells * per * args.steps / (ms / 1e3) / 1e9
    bpc = dispersive_bytes_per_cell(dims, 12, info["box"], 2, len(info["planes"]), len(info["freqs"]))
    bpc_ring = dispersive_bytes_per_cell(dims, 12, info["box"], 2, len(info["planes"]), len(info["freqs"]), "ring")
    avg = kern_ms / 1e3 / max(kern_n, 1)
    ach = bpc * cells / avg / 1e9
    _line(metric="Gcell-updates/s", value=value, unit="Gcell/s", steps=args.steps, warmup=args.warmup,
          ms_per_step=ms / args.steps, dtype="f32",
          config={"workload": "3d_dispersive_384x384x192: Drude + 2 Lorentz half-space metal, Si3N4 ridge, TFSF "
                              "plane wave (-z, Ex), two 64-frequency Ex DFT planes, 12-cell CPML",
                  "time_steps_per_step": per, "status": status, "l2": "inputs larger than L2",
                  "schedule": args.dispersive_schedule, "tuned_chunk": tuned},
          roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                    "peak_kind": peak_kind,
                    "traffic": _profile_value("fused_dispersive_384.json" if fused else "dispersive_384.json", dims,
                                              "dram_bytes_per_step"),
                    "bytes_per_cell_update": bpc, "frac_ring_model": bpc_ring * cells / avg / 1e9 / peak,
                    "bytes_per_cell_update_ring_model": bpc_ring,
                    "kernel": ("TFSF line + fused3_multi (H+E, CPML, TFSF corrections, ADE partial update) + "
                               "ade_pass3 (pole terms) per step" if fused else
                               "split H + E(ADE) + TFSF stencil per step"),
                    "avg_step_us": avg * 1e6},
          gpu_launches=eng.launch_count() - n0, clocks=clk)
    eng.close()


def run_sweep(args, cpu, peak, peak_kind):
    """Batched coupler sweep: one bench step = --designs designs x 4000 steps."""
    import torch

    from prismo_gb300 import sweep as S

    designs = [S.coupler_design(s) for s in range(args.designs)]
    layouts = [S.coupler_layout(d) for d in designs]
    B = S.BatchedFDTD2D(S.instances_for(layouts), S.sweep_freqs(S.NFREQ))
    variant = B.tuning()[0]
    tile = S.BatchedFDTD2D.variants()[variant]
    cells = sum(I.eps.shape[0] * I.eps.shape[1] for I in B.instances)
    B.close()
    runs = []
    clocks = ClockSampler(0)
    for q in range(max(args.warmup, 3) + args.steps):
        if q == max(args.warmup, 3):
            clocks.start()
        r = S.batched_sweep(designs, layouts=layouts, variant=variant)
        runs.append(r)
    clk = clocks.stop()
    timed = runs[-args.steps:]
    run_s = sum(r.run_seconds for r in timed) / args.steps
    e2e_s = sum(r.seconds for r in timed) / args.steps
    # end to end from the design list (layouts included) once more
    e2e = S.batched_sweep(designs, variant=variant)
    ser = S.serial_sweep(designs[:2])
    ser_k = S.serial_sweep(designs[:2], batch_route=False)
    err = float(np.abs(timed[-1].S[:2] - ser.S).max())
    # the batch kernel's roofline: unblocked 2D bytes per cell update (28 B + CPML edges)
    bpc = 28.0 + 16.0 * float(np.mean([(2 * S.CPML / I.eps.shape[0] + 2 * S.CPML / I.eps.shape[1])
                                       for I in S.instances_for(layouts)]))
    gcell = cells * S.STEPS / run_s / 1e9
    ach = gcell * bpc
    _line(metric="designs/s", value=args.designs / run_s, unit="designs/s", steps=args.steps, warmup=args.warmup,
          ms_per_step=run_s * 1e3, dtype="f32",
          config={"workload": f"batched 2D coupler sweep: {args.designs} designs (seeds 0..{args.designs - 1}), "
                              "Nx 400-1200, Ny 200-800, 20-cell CPML, 4000 steps, 4 ports x 64 frequencies, "
                              "plus one normalisation run per design",
                  "variant_tile_steps": tile, "gcell_per_s": gcell, "l2": "inputs larger than L2"},
          e2e={"value": args.designs / e2e.seconds, "unit": "designs/s", "h2d_bytes_per_step": int(
              sum(I.eps.nbytes for I in S.instances_for(layouts))), "d2h_bytes_per_step": int(
              e2e.S.size * 16), "api": "prismo_gb300.sweep.batched_sweep (design list in, S-parameters out)"},
          serial_designs_per_s=ser.designs_per_s, batched_vs_serial=(args.designs / e2e.seconds) / ser.designs_per_s,
          serial_per_step_kernels_designs_per_s=ser_k.designs_per_s,
          batched_vs_serial_per_step_kernels=(args.designs / e2e.seconds) / ser_k.designs_per_s,
          max_abs_S_batched_vs_serial=err,
          roofline={"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                    "peak_kind": peak_kind, "traffic": None, "bytes_per_cell_update": bpc,
                    "kernel": f"batch2d_pass<{tile[0]},{tile[1]},{tile[2]}> (unblocked bytes; K steps per pass)"},
          cpu_baseline=cpu, gpu_launches=timed[-1].launches, clocks=clk)


def run_surrogate(args, cpu):
    """Train the 4-member ensemble on 4096 batched-FDTD designs, then run the
    surrogate + FDTD-fallback pipeline on 256 held-out designs."""
    import torch

    from prismo_gb300 import surrogate as Su
    from prismo_gb300 import sweep as S

    t0 = time.perf_counter()
    train = [S.coupler_design(s) for s in range(4096)]
    test = [S.coupler_design(s) for s in range(10000, 10256)]
    Str = np.concatenate([S.batched_sweep(train[q:q + 1024]).S for q in range(0, 4096, 1024)])
    ref = S.batched_sweep(test)
    t_data = time.perf_counter() - t0
    E = Su.Ensemble()
    E.fit(train, Str, epochs=Su.EPOCHS)
    # gate calibration on designs held out from training and from the test set
    calib = [S.coupler_design(s) for s in Su.CALIB_SEEDS]
    t0 = time.perf_counter()
    E.calibrate(calib, np.concatenate([S.batched_sweep(calib[q:q + 512]).S for q in range(0, len(calib), 512)]))
    t_calib = time.perf_counter() - t0
    res = Su.run_pipeline(E, test)
    err = Su.s_error(res.S, ref.S)
    acc = res.accepted
    ser = S.serial_sweep(test[:4])
    ser_k = S.serial_sweep(test[:4], batch_route=False)
    # inference on a batch of 8192 queries (host features + device forward + re-embedding)
    q = [S.coupler_design(s) for s in range(20000, 20000 + 8192)]
    E.predict(q[:64])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, spread_q, _ = E.predict(q)
    t_inf = time.perf_counter() - t0
    xd = torch.as_tensor(E._features(Su.inputs(q)), device="cuda")

    def forward_ms():
        for _ in range(3):
            E.forward_raw(xd)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(20):
            E.forward_raw(xd)
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / 20

    E.set_tensor_path(False)
    fwd_ms_mma = forward_ms()
    E.set_tensor_path(True)
    fwd_ms = forward_ms()
    dims = E.dims
    flops = E.members * 8192 * 2 * (32 * dims[1] + dims[1] * dims[2] + dims[2] * dims[3] + dims[3] * dims[4])
    r_fdtd = len(test) / ref.seconds
    frac = float(acc.mean())
    dps_8192 = 8192 / (t_inf + (1 - frac) * 8192 / r_fdtd)
    _line(metric="designs/s", value=res.designs_per_s, unit="designs/s", steps=1, warmup=0,
          ms_per_step=res.seconds * 1e3, dtype="bf16 (f32 accumulate)",
          config={"workload": "surrogate + batched-FDTD fallback on 256 held-out couplers (seeds 10000-10255); "
                              "4-member ensemble 31-256-256-256-512 SiLU (3 geometry floats + per-member random "
                              "Fourier embedding) trained on 4096 batched-FDTD designs (seeds 0-4095)",
                  "error_bar": Su.THRESHOLD, "gate": E.calibration, "calibration_seconds": t_calib,
                  "epochs": Su.EPOCHS, "train_seconds": E.train_seconds,
                  "train_steps": E.train_steps, "data_seconds": t_data},
          accepted=int(acc.sum()), accepted_fraction=frac,
          err_rms_answered={"median": float(np.median(err[acc])) if acc.any() else None,
                            "p90": float(np.percentile(err[acc], 90)) if acc.any() else None,
                            "max": float(err[acc].max()) if acc.any() else None,
                            "frac_le_1e-3": float(np.mean(err[acc] <= 1e-3)) if acc.any() else None},
          err_rms_all_max=float(err.max()),
          batched_fdtd_designs_per_s=r_fdtd, serial_designs_per_s=ser.designs_per_s,
          pipeline_vs_serial=res.designs_per_s / ser.designs_per_s,
          serial_per_step_kernels_designs_per_s=ser_k.designs_per_s,
          pipeline_vs_serial_per_step_kernels=res.designs_per_s / ser_k.designs_per_s,
          inference={"queries": 8192, "seconds": t_inf, "designs_per_s": 8192 / t_inf,
                     "accept_fraction": float(np.mean(E.gate(q, spread_q))),
                     "device_forward_ms": fwd_ms, "device_tflops": flops / (fwd_ms * 1e-3) / 1e12,
                     "device_forward_ms_mma_sync": fwd_ms_mma,
                     "pipeline_designs_per_s_8192": dps_8192,
                     "pipeline_vs_serial_8192": dps_8192 / ser.designs_per_s},
          e2e={"value": res.designs_per_s, "unit": "designs/s", "h2d_bytes_per_step": len(test) * 12,
               "d2h_bytes_per_step": len(test) * 512 * 4, "api": "prismo_gb300.surrogate.run_pipeline"},
          cpu_baseline=cpu, gpu_launches=E.launches)


def run_mlp(args):
    """The surrogate ensemble's forward pass alone: 4 members x 8192 query rows
    through 31-256-256-256-512 (bf16 hi/lo activations, float32 accumulation), on
    the tcgen05 path and on the mma.sync path; one bench step = one forward."""
    import torch

    from prismo_gb300 import surrogate as Su

    E = Su.Ensemble()
    B = 8192
    rng = np.random.default_rng(0)
    E.set_params(rng.normal(0.0, 0.05, E.params().shape))  # every layer non-zero
    x = torch.tensor(rng.standard_normal((E.members, B, E.dims[0])).astype(np.float32), device="cuda")
    dims = E.dims
    flops = E.members * B * 2 * (32 * dims[1] + dims[1] * dims[2] + dims[2] * dims[3] + dims[3] * dims[4])

    def timed(tc):
        E.set_tensor_path(tc)
        for _ in range(max(args.warmup, 3)):
            E.forward_raw(x)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n0 = E.launches
        ev0.record()  # the ensemble launches on torch's current stream
        for _ in range(args.steps):
            E.forward_raw(x)
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / args.steps, (E.launches - n0) // max(args.steps, 1)

    ms_mma, _ = timed(False)
    ms_tc, launches = timed(True)
    y_tc = E.forward_raw(x)
    E.set_tensor_path(False)
    y_mma = E.forward_raw(x)
    rel = float((y_tc - y_mma).norm() / y_mma.norm().clamp_min(1e-30))

    # training steps (forward, loss gradient, backward products, Adam): the
    # surrogate's 256-design batches, and 4096-design batches where the backward
    # products fill the GPU
    def timed_train(tc, Bt, reps=30):
        xt = x[:, :Bt].contiguous()
        tt = torch.zeros((E.members, Bt, dims[-1]), dtype=torch.float32, device="cuda")
        E.set_tensor_path(tc)
        for _ in range(5):
            E.train_step_raw(xt, tt, 1e-6)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(reps):
            E.train_step_raw(xt, tt, 1e-6)
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    train = {}
    for Bt in (256, 4096):
        fl = 3 * E.members * Bt * 2 * (32 * dims[1] + dims[1] * dims[2] + dims[2] * dims[3] + dims[3] * dims[4])
        t = {k: timed_train(v, Bt) for k, v in (("mma_sync", False), ("tcgen05", True), ("auto", "auto"))}
        train[f"batch_{Bt}"] = {**{f"ms_{k}": v for k, v in t.items()},
                                "tflops_tcgen05": fl / (t["tcgen05"] * 1e-3) / 1e12}
    E.set_tensor_path("auto")
    status = E.status()
    E.close()
    _line(metric="TFLOP/s", value=flops / (ms_tc * 1e-3) / 1e12, unit="TFLOP/s", steps=args.steps,
          warmup=args.warmup, ms_per_step=ms_tc, dtype="bf16 (f32 accumulate)",
          config={"workload": "surrogate forward: 4 members x 8192 rows, 31-256-256-256-512 SiLU, bf16 hi/lo "
                              "activations", "status": status, "tcgen05_vs_mma_sync_rel": rel},
          mma_sync_ms_per_step=ms_mma, gpu_launches=launches, train_step_per_member_batch=train)


if __name__ == "__main__":
    main()
