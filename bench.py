#!/usr/bin/env python
"""Throughput of the Fluid2d time step on GB300: cell-steps/s per RK3 step.

Headline workload: Euler 2D decaying turbulence on a doubly periodic
1024 x 1024 unit box, random-phase vorticity with E(k) ~ k^3 exp(-(k/10)^2),
rms 1 (seeded synthetic data: the reference publishes no dataset), 5th-order
upwind advection, RK3-SSP, multigrid Poisson inversion (two V-cycles per
inverting stage, full F-cycle solve after every step), float64, fixed dt from
CFL 0.8 on the initial max|u|.

One bench "step" is one iteration of the reference's time loop
(core/fluid2d.py:237-268): set_dt, model.step (3 RK stages + solve),
diagnostics.  value = interior cells x steps / device time.  The working set
(state, RK tendencies, stage states, multigrid hierarchy, ~0.3 GB) is larger
than the 129 MB L2, so no flush is needed between steps.

The same JSON line carries the other named workloads under "configs":
the closed 128^2 dipole (200 steps, with its CPU path on one core and on
every core), the 2048x512 Boussinesq shear layer (1000 steps of the float64
and the mixed form, the mixed form's error every 100 steps), the
96-instance batched ensemble (100 steps) and a sample of the served stream
(requests with U[50, 500] steps, Poisson arrivals at 40/s).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --profile-step [...]      one NVTX-bracketed step for ncu

--impl reference times the reference's own CPU implementation of the path
(its Fortran kernels restated in C, driven by a restatement of its Python
sequencing -- the reference's Fortran cannot be compiled here) on all the
host's cores, each core stepping its own copy of the workload.
Under torchrun (N > 1) every rank steps an independent replica (the path
has no data-path collective); value sums the replicas.
"""
import argparse
import os as _os
# independent simulations overlap on up to 32 hardware queues
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-steps/s per RK3 step"
UNIT = "cell-steps/s"
NX = NY = 1024
WORKLOAD = "euler-decaying-turbulence-1024x1024-perio-fp64"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=NX, help="grid side (default 1024)")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--dipole-steps", type=int, default=200)
    ap.add_argument("--shear-steps", type=int, default=1000)
    ap.add_argument("--shear-cpu-steps", type=int, default=5)
    ap.add_argument("--ensemble-steps", type=int, default=100)
    ap.add_argument("--ensemble-cpu-steps", type=int, default=3)
    ap.add_argument("--served-requests", type=int, default=200)
    ap.add_argument("--served-slots", type=int, default=16,
                    help="simulations running at once at most (0: the budget alone decides)")
    ap.add_argument("--served-chunk", type=int, default=16,
                    help="steps queued at a time for each served simulation")
    ap.add_argument("--alone-steps", type=int, default=20,
                    help="steps timed per request when run alone (the rest extrapolated)")
    ap.add_argument("--only", default="",
                    help="comma list of extra measurements to run: "
                         "mixed,dipole,shear,ensemble,served (default all; 'none')")
    return ap.parse_args(argv)


def wanted(a, key):
    if not a.only:
        return True
    return key in a.only.split(",")


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def host_info():
    """CPU model and logical core count of this host."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k = line.split(":")[0].strip().lower()
                if k in ("model name", "cpu model", "hardware") and ":" in line:
                    model = line.split(":", 1)[1].strip()
                    break
    except OSError:
        pass
    if not model:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for line in out.splitlines():
                if line.lower().startswith("model name"):
                    model = line.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    import platform
    return {"cpu": model or platform.processor() or "unknown", "arch": platform.machine(),
            "nproc": os.cpu_count() or 1}


# ------------------------------------------------------------------ clocks
class ClockSampler(object):
    """nvidia-smi samples of SM clock and throttle reasons during timing."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU side
def _workload(kind, n=None, index=None):
    from fluid2d_gb300 import workloads as W
    if kind == "turbulence":
        return W.turbulence(n, n, seed=2)
    if kind == "dipole":
        return W.dipole(128, 128)
    if kind == "shear":
        return W.shear(2048, 512)
    if kind == "ensemble":
        return W.ensemble(96, seed=4)[index]
    raise ValueError(kind)


def _cpu_worker(args):
    """Step the oracle (the reference's CPU path restated, timing build) on
    one workload, for `steps` steps or until `budget` seconds have passed."""
    kind, n, index, budget, steps = args
    os.environ["F2D_ORACLE_VARIANT"] = "timing"
    sys.path.insert(0, ROOT)
    from oracle import stepper
    wl = _workload(kind, n, index)
    p, M = stepper.from_workload(wl)
    dt = 0.8 * min(M.grid.dx, M.grid.dy) / M.diags["maxspeed"]
    t0 = time.perf_counter()
    done = 0
    t = 0.
    while True:
        t = stepper.run(M, p, 1, dt, t=t)
        done += 1
        el = time.perf_counter() - t0
        if (steps and done >= steps) or (not steps and el >= budget):
            break
    return done, time.perf_counter() - t0, wl["nx"] * wl["ny"]


# float64 FMA throughput of a GB300 of this machine (independent DFMA chains on
# every SM, CUDA events), used only if the live measurement (f2d_fp64_peak)
# fails: the FP64-ALU roofline of the float64 kernels
FP64_PEAK_TFLOPS = 1.20
SMOOTH_DRAM_BYTES_PER_POINT = (20118016 + 0 + 20078848 + 0) / 1060900.


def cpu_run(jobs, cores):
    """Run oracle jobs (see _cpu_worker) on `cores` processes; returns
    cell-steps/s over the slowest process's wall time and the per-job
    results.  The pool is started with 'spawn'."""
    from oracle import oracle
    oracle.build()
    if cores == 1 and len(jobs) == 1:
        res = [_cpu_worker(jobs[0])]
    else:
        import multiprocessing as mp
        with mp.get_context("spawn").Pool(cores) as pool:
            res = pool.map(_cpu_worker, jobs)
    total = sum(d * c for d, _, c in res)
    if cores == 1:
        wall = sum(w for _, w, _ in res)
    elif len(jobs) <= cores:
        wall = max(w for _, w, _ in res)  # one job per process, all at once
    else:
        # more jobs than processes: the stepping time shared evenly over the
        # cores (set-up between jobs not counted) -- the CPU's best case
        wall = sum(w for _, w, _ in res) / cores
    return total / wall, res


def cpu_baseline(n, budget, cores):
    """Cell-steps/s of the oracle path on `cores` host processes, each on its
    own copy of the n x n turbulence workload for about `budget` seconds."""
    val, res = cpu_run([("turbulence", n, None, budget, 0)] * cores, cores)
    steps = sum(d for d, _, _ in res)
    if cores == 1:
        return val, "1 process, %d steps of the %dx%d workload in %.1f s" % (
            steps, n, n, res[0][1])
    return val, ("%d processes, each stepping its own %dx%d copy for ~%.0f s (%d steps in total)"
                 % (cores, n, n, budget, steps))


def cpu_descr(cores, sample, val, host):
    return {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
            "build": "C restatement of the Fortran, gcc -O3 -ffp-contract=fast (FMA)",
            "host_cpu": host["cpu"], "host_nproc": host["nproc"]}


def max_over_ranks(value, world, device="cuda"):
    """The largest `value` over the ranks of the process group (every rank
    gets it); the value itself when there is one rank."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(a, rank, world):
    if rank != 0:
        return
    host = host_info()
    cores = host["nproc"]
    K, W = a.steps, a.warmup
    # the whole --steps/--warmup run is one bounded sample per core
    val, sample = cpu_baseline(a.n, a.cpu_sample_s, cores)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT,
            "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "euler-decaying-turbulence-%dx%d-perio-fp64"
                                            % (a.n, a.n), "nx": a.n, "ny": a.n},
            "cpu_baseline": cpu_descr(cores, sample, val, host),
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU side
def run_ours(a, rank, world, local):
    import numpy as np
    import torch
    import torch.distributed as dist
    from fluid2d_gb300 import engine, workloads as W
    from fluid2d_gb300._lib import so_path

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    n = a.n
    wl = W.turbulence(n, n, seed=2)
    M = engine.from_workload(wl, dt=1e-3)
    M.set_psi_from_vorticity()
    d0 = M.diagnostics()
    dt = 0.8 * min(M.dx, M.dy) / d0["maxspeed"]
    M.set_dt(dt)
    s0 = M.var.state.clone()
    # the coarse-CTA switch level that times fastest on this grid (the
    # state it advanced is put back; results do not depend on the choice)
    from fluid2d_gb300.autotune import tune_coarse_level, tune_level_tiles
    tune_coarse_level(M, steps=3, warmup=1)
    # and the level kernels' tile shape and block size (process-wide)
    tiles, _ = tune_level_tiles(M, steps=3, warmup=1)
    M.var.state.copy_(s0)
    M.diagnostics()
    stream = torch.cuda.Stream()
    # warm-up: capture the step graph and run W steps
    with torch.cuda.stream(stream):
        M.run(a.warmup, graph=True)
    stream.synchronize()
    kernels_per_step = M.graph_kernels()

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- timed region: K graph replays, device time with CUDA events
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record(stream)
            M.run(a.steps, graph=True)
            e1.record(stream)
        e1.synchronize()
        torch.cuda.synchronize()
        barrier()
    ms = max_over_ranks(e0.elapsed_time(e1), world)
    ms_step = ms / a.steps
    value = world * n * n * a.steps / (ms * 1e-3)
    nite, res, st = M.solve_stats()
    diags = M.read_diags()
    nlevs, coarse_level, coarse_points = M.nlevs, M.coarse_level, M.coarse_operator()

    # ---- roofline of the dominant kernel (the finest-level smoother, timed
    # with CUDA events around every call inside the replayed step graph)
    nprobe, probe_ms = 0, 0.
    try:
        M.probe(True)
        with torch.cuda.stream(stream):
            M.run(3, graph=True)
        stream.synchronize()
        nprobe, probe_ms = M.probe()
        M.probe(False)
    except Exception as exc:  # keep the bench line even if the probe fails
        print("probe failed: %s" % exc, file=sys.stderr)
    roofline = smoother_roofline(n, probe_ms, nprobe)

    # ---- e2e through the public API with host buffers: every step uploads
    # the state (Var.state's layout) from pinned memory, steps, reads it back
    # (Model.run_host: one call a step; the copies and the step are one graph)
    state_host = torch.empty(M.var.state.shape, dtype=torch.float64).pin_memory()
    state_host.copy_(M.var.state.cpu())
    h2d = d2h = state_host.numel() * 8
    with torch.cuda.stream(stream):
        for _ in range(2):
            M.run_host(1, state_host)
        stream.synchronize()
        barrier()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(a.e2e_steps):
            M.run_host(1, state_host)
        f1.record(stream)
        f1.synchronize()
    e2e_ms = max_over_ranks(f0.elapsed_time(f1), world)
    e2e_val = world * n * n * a.e2e_steps / (e2e_ms * 1e-3)
    del M
    torch.cuda.synchronize()

    # the other workloads tune their own launch structure; the level kernels
    # go back to their default tiles and block sizes
    try:
        from fluid2d_gb300 import _lib as _l
        _l.lib().f2d_set_level_tiles(0)
        _l.lib().f2d_set_level_threads(0)
    except Exception as exc:
        print("level tiles reset failed: %s" % exc, file=sys.stderr)
    host = host_info()
    extra = {}
    if rank == 0:
        todo = [("mixed", lambda: bench_mixed(engine, wl, dt, s0, a, stream, world)),
                ("dipole", lambda: bench_dipole(a, host)),
                ("shear", lambda: bench_shear(a, host)),
                ("ensemble", lambda: bench_ensemble(a, host)),
                ("served", lambda: bench_served(a))]
        for key, fn in todo:
            if not wanted(a, key):
                continue
            try:
                extra[key] = fn()
            except Exception as exc:
                import traceback
                traceback.print_exc()
                print("%s failed: %s" % (key, exc), file=sys.stderr)
            torch.cuda.synchronize()
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    cpu = None
    if not a.no_cpu_baseline:
        v, sample = cpu_baseline(n, a.cpu_sample_s, 1)
        cpu = cpu_descr(1, sample, v, host)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded random-phase vorticity, E(k)~k^3 exp(-(k/10)^2), rms 1",
        "config": {"workload": "euler-decaying-turbulence-%dx%d-perio-fp64" % (n, n),
                   "nx": n, "ny": n, "precision": "fp64", "cuda_graph": True,
                   "multigrid_levels": nlevs, "coarse_cta_from_level": coarse_level,
                   "coarse_operator_points": coarse_points,
                   "level_tiles": {"cta_target": tiles[0], "one_pass_threads": tiles[1]},
                   "solve_iterations_last_step": nite, "solve_residual_last_step": res,
                   "dt": dt, "maxspeed": diags.get("maxspeed"),
                   "l2": "working set > L2 (state, tendencies, hierarchy ~0.3 GB); no flush",
                   "parallelism": "replicas" if world > 1 else "single"},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": a.e2e_steps},
        "gpu_launches": kernels_per_step * a.steps,
        "clocks": clk.summary(),
        "host": host,
        "mixed": extra.get("mixed"),
        "configs": {"dipole_128_closed_fp64": extra.get("dipole"),
                    "shear_2048x512_boussinesq": extra.get("shear"),
                    "ensemble_96": extra.get("ensemble"),
                    "served_stream": extra.get("served")},
        "libraries": [os.path.basename(so_path("product"))],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def smoother_roofline(n, probe_ms, nprobe):
    """The finest-level smoother (one smoothtwicewitha call: the two float64
    Jacobi sweeps of core/gmg/fortran_multigrid.f90:2-127) against its bound,
    the float64 pipe: 19 flops per point per sweep (1 mul, 7 fma, 1 sub,
    1 mul, 1 fma), two sweeps per call, over the call's mean CUDA-event
    duration inside the replayed step graph (the call after a coarse
    correction also holds its prolongation); peak = float64 FMA chains
    measured live on this GPU (f2d_fp64_peak).  The flops are the
    algorithm's: the column form (k_sweepc) executes fewer float64
    instructions for the same sweep.  Beside it, the same call
    against HBM: x, b read, x written (8 B each) and the mask (1 B) = 25 B
    per point, with the DRAM traffic of an ncu capture of the same kernels."""
    pts = (n + 6) * (n + 6)
    fp64_flops = 2 * 19 * pts
    achieved = fp64_flops / (probe_ms * 1e-3) / 1e12 if probe_ms > 0 else None
    fp64_peak, fp64_src = FP64_PEAK_TFLOPS, "fallback: earlier FMA-chain measurement on this pool"
    try:
        import ctypes as _ct
        from fluid2d_gb300 import _lib as _l
        _v = _ct.c_double()
        if _l.lib().f2d_fp64_peak(_ct.byref(_v)) == 0 and _v.value > 0:
            fp64_peak, fp64_src = _v.value, "measured live: f2d_fp64_peak (float64 FMA chains)"
    except Exception as exc:
        print("fp64 peak failed: %s" % exc, file=sys.stderr)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except (OSError, ValueError):
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    alg_bytes = 25 * pts
    hbm = alg_bytes / (probe_ms * 1e-3) / 1e9 if probe_ms > 0 else None
    # dram__bytes_read.sum + dram__bytes_write.sum of one call per grid point
    # (ncu capture of k_sweepc, the column form, in the 1024^2 turbulence step)
    traffic = SMOOTH_DRAM_BYTES_PER_POINT * pts
    return {"kernel": "finest-level smoother (smoothtwicewitha: the two float64 sweeps)",
            "bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
            "frac": (achieved / fp64_peak) if achieved else None,
            "flops_per_launch": fp64_flops, "peak_source": fp64_src,
            "traffic": traffic, "alg_bytes_per_launch": alg_bytes,
            "launches_probed": nprobe, "avg_launch_ms": probe_ms,
            "hbm": {"achieved": hbm, "peak": hbm_peak, "unit": "GB/s",
                    "frac": (hbm / hbm_peak) if hbm else None,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}}


def _timed_graph(model, steps, stream):
    """ms of `steps` graph replays of the model's step (CUDA events)."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        model.run(steps, graph=True)
        e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def _rel(a, b):
    import numpy as np
    nb = float(np.sqrt((b ** 2).sum()))
    mb = float(np.abs(b).max())
    return {"rel_l2": float(np.sqrt(((a - b) ** 2).sum())) / nb if nb > 0 else None,
            "rel_linf": float(np.abs(a - b).max()) / mb if mb > 0 else None}


def bench_mixed(engine, wl, dt, s0, a, stream, world):
    """Throughput of the mixed form on the headline workload, and its
    single-step error against the float64 oracle from the oracle's state
    (per field, relative L2 and L-inf)."""
    import torch
    from oracle import stepper
    n = wl["nx"]
    from fluid2d_gb300 import _lib as lib
    from fluid2d_gb300.autotune import tune_coarse_level, tune_level_tiles
    L = lib.lib()
    # the level tiles are process settings: tuned for this model, then put
    # back for the measurements that follow
    prev = (L.f2d_set_level_tiles(-2), L.f2d_set_level_threads(-1))
    Mm = engine.from_workload(wl, dt=dt, precision="mixed")
    Mm.var.state.copy_(s0)
    Mm.diagnostics()
    tune_coarse_level(Mm, steps=3, warmup=1)
    tiles, _ = tune_level_tiles(Mm, steps=3, warmup=1)
    Mm.var.state.copy_(s0)
    Mm.diagnostics()
    with torch.cuda.stream(stream):
        Mm.run(a.warmup, graph=True)
    stream.synchronize()
    ms = _timed_graph(Mm, a.steps, stream)
    nite, res, st = Mm.solve_stats()
    del Mm
    L.f2d_set_level_tiles(prev[0])
    L.f2d_set_level_threads(prev[1])
    # one step of the mixed form and of the oracle from the oracle's state
    p, O = stepper.from_workload(wl)
    odt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
    B = engine.from_workload(wl, dt=odt, precision="mixed")
    B.var.state.copy_(torch.from_numpy(O.state).cuda())
    B.diagnostics()
    stepper.run(O, p, 1, odt)
    B.run(1)
    got = B.var.state.cpu().numpy()
    err = {}
    for k, nm in enumerate(B.var.varname_list):
        if abs(O.state[k]).max() > 0:
            err[nm] = _rel(got[k], O.state[k])
    return {"value": world * n * n * a.steps / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms / a.steps, "dtype": "f32 fluxes and multigrid, f64 defect "
            "correction, RK accumulation and diagnostics",
            "single_step_error_vs_f64_oracle": err, "solve_iterations_last_step": nite,
            "solve_residual_last_step": res,
            "level_tiles": {"cta_target": tiles[0], "one_pass_threads": tiles[1]}}


def _device_start(engine, wl, **kw):
    """A model of the workload with psi inverted and dt set on the device
    (dt = 0.8 min(dx, dy) / maxspeed), and a copy of its state."""
    import torch
    M = engine.from_workload(wl, dt=1e-3, **kw)
    M.set_psi_from_vorticity()
    dt = 0.8 * min(M.dx, M.dy) / M.diagnostics()["maxspeed"]
    M.set_dt(dt)
    s0 = M.var.state.clone()
    torch.cuda.synchronize()  # the copy is complete before other streams step M
    return M, dt, s0


def _oracle_start(engine, stepper, wl, **kw):
    """The parity check's start: the oracle's model of the workload and a
    GPU model holding the oracle's state and dt."""
    import torch
    p, O = stepper.from_workload(wl)
    dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
    G = engine.from_workload(wl, dt=dt, **kw)
    G.var.state.copy_(torch.from_numpy(O.state).cuda())
    G.diagnostics()
    return p, O, dt, G


def bench_dipole(a, host):
    """Euler dipole, closed 128x128, 200 steps (the reference's CPU-runnable
    case): the float64 GPU path from its own initial state (psi inverted on
    the device), timed as a graph; parity: the GPU path and the oracle both
    from the oracle's state, compared after the 200 steps, which on one core
    also give the CPU rate; the CPU path on every core (one copy each) gives
    the host's aggregate rate."""
    import torch
    from fluid2d_gb300 import engine, workloads as W
    from oracle import stepper
    steps = a.dipole_steps
    wl = W.dipole(128, 128)
    stream = torch.cuda.Stream()
    G, dt, s0 = _device_start(engine, wl)
    with torch.cuda.stream(stream):
        G.run(5, graph=True)  # capture, warm up
    stream.synchronize()
    G.var.state.copy_(s0)
    G.diagnostics()
    ms = _timed_graph(G, steps, stream)
    del G
    p, O, odt, P = _oracle_start(engine, stepper, wl)
    with torch.cuda.stream(stream):
        P.run(steps, graph=True)
    stream.synchronize()
    final = P.var.state.cpu().numpy()
    stepper.run(O, p, steps, odt)
    parity = {nm: _rel(final[k], O.state[k])["rel_linf"]
              for k, nm in enumerate(P.var.varname_list) if nm in ("vorticity", "psi", "u", "v")}
    del P
    one, res1 = cpu_run([("dipole", None, None, 0, steps)], 1)
    cores = host["nproc"]
    allc, _ = cpu_run([("dipole", None, None, 0, steps)] * cores, cores)
    value = 128 * 128 * steps / (ms * 1e-3)
    return {"value": value, "unit": UNIT, "ms_per_step": ms / steps, "steps": steps,
            "precision": "fp64", "dt": dt,
            "parity_rel_linf_after_%d_steps_vs_oracle" % steps: parity,
            "cpu_baseline_1core": cpu_descr(1, "the %d steps on one core" % steps, one, host),
            "cpu_baseline_all_cores": cpu_descr(cores, "%d copies, one per core, %d steps each"
                                                % (cores, steps), allc, host),
            "gpu_vs_cpu_1core": value / one, "gpu_vs_cpu_all_cores": value / allc}


def bench_shear(a, host):
    """Boussinesq shear layer, 'xchannel' 2048x512, Ri = 0.1: 1000 steps of
    the float64 form and of the mixed form from the same state, each timed
    (graph replays, 100 steps at a time), with the mixed form's per-field
    error against the float64 path every 100 steps.  The float64 GPU path is
    compared with the oracle over the first --shear-cpu-steps steps, which
    also time the CPU path on one core (rate extrapolated to the run)."""
    import numpy as np
    import torch
    from fluid2d_gb300 import engine, workloads as W
    from oracle import stepper
    wl = W.shear(2048, 512)
    cells = 2048 * 512
    stream = torch.cuda.Stream()
    # parity of the float64 form with the oracle over the first steps, both
    # from the oracle's state
    p, O, odt, P = _oracle_start(engine, stepper, wl)
    ncpu = a.shear_cpu_steps
    P.run(ncpu)
    t0 = time.perf_counter()
    stepper.run(O, p, ncpu, odt)
    t_oracle = time.perf_counter() - t0
    got = P.var.state.cpu().numpy()
    parity = {nm: _rel(got[k], O.state[k])["rel_linf"]
              for k, nm in enumerate(P.var.varname_list)
              if nm in ("vorticity", "psi", "u", "v", "buoyancy")}
    del P, O
    # the timed runs start from the state prepared on the device
    A, dt, s0 = _device_start(engine, wl)
    B = engine.from_workload(wl, dt=dt, precision="mixed")
    # 1000 steps of each form, 100 at a time
    for M in (A, B):
        M.var.state.copy_(s0)
        M.diagnostics()
        with torch.cuda.stream(stream):
            M.run(1, graph=True)  # capture
        stream.synchronize()
        M.var.state.copy_(s0)
        M.diagnostics()
    every = 100
    ms = {"fp64": 0., "mixed": 0.}
    rows = []
    for k in range(every, a.shear_steps + 1, every):
        ms["fp64"] += _timed_graph(A, every, stream)
        ms["mixed"] += _timed_graph(B, every, stream)
        fa, fb = A.var.state.cpu().numpy(), B.var.state.cpu().numpy()
        row = {"step": k}
        for q, nm in enumerate(A.var.varname_list):
            if nm in ("vorticity", "psi", "u", "v", "buoyancy"):
                row[nm] = _rel(fb[q], fa[q])
        iu, iv = A.var.varname_list.index("u"), A.var.varname_list.index("v")
        nrm = float(np.sqrt((fa[iu] ** 2).sum() + (fa[iv] ** 2).sum()))
        row["velocity_rel_l2"] = float(np.sqrt(((fb[iu] - fa[iu]) ** 2).sum()
                                               + ((fb[iv] - fa[iv]) ** 2).sum())) / nrm
        rows.append(row)
    n = a.shear_steps
    cpu = cells * ncpu / t_oracle
    return {"fp64": {"value": cells * n / (ms["fp64"] * 1e-3), "unit": UNIT,
                     "ms_per_step": ms["fp64"] / n},
            "mixed": {"value": cells * n / (ms["mixed"] * 1e-3), "unit": UNIT,
                      "ms_per_step": ms["mixed"] / n},
            "steps": n, "dt": dt, "gravity": wl["gravity"], "richardson": 0.1,
            "parity_fp64_rel_linf_vs_oracle_after_%d_steps" % ncpu: parity,
            "mixed_error_vs_fp64_every_100_steps": rows,
            "cpu_baseline_1core": cpu_descr(1, "first %d steps of the oracle (parity build) "
                                            "on one core, rate extrapolated to the run" % ncpu,
                                            cpu, host),
            "gpu_fp64_vs_cpu_1core": cells * n / (ms["fp64"] * 1e-3) / cpu}


def _structure(choice):
    off, groups, policy = choice
    lev = "coarse switch first+%d" % off
    if groups == 0:
        return "streams, " + lev
    return "batched groups=%d policy=%d, %s" % (groups, policy, lev)


def bench_ensemble(a, host):
    """Config: 96 independent Euler instances (sides log-uniform 64-768,
    multiples of 64, islands, 3-12 vortices; seed 4), 100 steps.  Batched =
    the launch structure the autotuner picks (fluid2d_gb300.autotune.
    tune_ensemble): groups of instances whose steps are merged into one
    launch per kernel, one graph per group on its own stream, or every
    instance's own step graph replayed on 32 streams; comparators = the plain
    float64 path one instance at a time, and the CPU path with the 96
    instances spread over every host core (a few steps each)."""
    import torch
    from fluid2d_gb300 import engine, workloads as W
    from fluid2d_gb300.autotune import tune_ensemble
    wls = W.ensemble(96, seed=4)
    cells = sum(w["nx"] * w["ny"] for w in wls)
    steps = a.ensemble_steps
    out = {"instances": len(wls), "cells": cells, "steps": steps}
    for prec in ("mixed", "fp64"):
        E = engine.ensemble_from_workloads(wls, precision=prec, nstreams=32)
        choice, times = tune_ensemble(E, steps=3, warmup=1)
        E.run(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        E.run(steps)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        failed = E.retire_failed()
        out[prec + "_batched"] = {"cell_steps_per_s": cells * steps / (ms * 1e-3),
                                  "ms_per_ensemble_step": ms / steps,
                                  "launch_structure": _structure(choice),
                                  "failed_instances": len(failed),
                                  "tuning_ms_per_step": {_structure(k): round(v, 3)
                                                         for k, v in times.items()}}
        E.free_batch()
        del E
        torch.cuda.synchronize()
    # one at a time, plain float64
    tot_ms = 0.
    nst = 10
    s = torch.cuda.Stream()
    for w in wls:
        E = engine.ensemble_from_workloads([w], precision="fp64", nstreams=1)
        m = E.models[0]
        with torch.cuda.stream(s):
            m.run(1, graph=True)
            s.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            m.run(nst, graph=True)
            e1.record(s)
            e1.synchronize()
        tot_ms += e0.elapsed_time(e1) / nst
        del E, m
    out["fp64_one_at_a_time"] = {"cell_steps_per_s": cells / (tot_ms * 1e-3),
                                 "ms_per_ensemble_step": tot_ms, "steps_timed_each": nst}
    out["mixed_batched_vs_fp64_one_at_a_time"] = (
        out["mixed_batched"]["cell_steps_per_s"] / out["fp64_one_at_a_time"]["cell_steps_per_s"])
    cores = host["nproc"]
    k = a.ensemble_cpu_steps
    cpu, _ = cpu_run([("ensemble", None, i, 0, k) for i in range(len(wls))], cores)
    out["cpu_baseline"] = cpu_descr(cores, "the 96 instances over %d processes, %d steps each "
                                    "(stepping time shared evenly over the cores)" % (cores, k),
                                    cpu, host)
    out["mixed_batched_vs_cpu"] = out["mixed_batched"]["cell_steps_per_s"] / cpu
    return out


def bench_served(a):
    """Config: served stream with Poisson arrivals at 40/s, 70 % Euler /
    30 % Boussinesq, sides 128-2048 (multiples of 128), HBM budget 150 GB,
    steps U[50, 500].  Sample: the first --served-requests requests of the
    2000-request stream, served in the mixed form with every admitted
    simulation running free on its own stream (chunks of --served-chunk
    steps), at two slot counts: --served-slots (throughput) and 4
    (latency).  Comparator: the same requests one at a time on the plain
    float64 path, each timed over --alone-steps steps after its graph capture
    (a fixed-dt step costs the same every step; the request's time is its
    step count times that)."""
    from fluid2d_gb300 import serve, workloads as W
    full = 2000
    stream = W.served_stream(count=a.served_requests, rate=40., seed=5)
    alone = serve.run_one_at_a_time(stream, precision="fp64", timed_steps=a.alone_steps)
    out = {"sample": "%d of the %d requests (%.0f %%), steps U[50,500], sides 128-2048, "
                     "70%% Euler / 30%% Boussinesq, Poisson 40/s, budget 150 GB"
                     % (len(stream), full, 100. * len(stream) / full),
           "fp64_one_at_a_time": alone}
    for key, slots in (("served_mixed_free_running", a.served_slots),
                       ("served_mixed_free_running_4_slots", 4)):
        srv = serve.Server(150e9, precision="mixed", nstreams=32, max_active=slots or None)
        m = srv.run_free(stream, chunk=a.served_chunk)
        m["slots"] = slots or None
        m["chunk_steps"] = a.served_chunk
        m["peak_active"] = srv.peak_active
        m["peak_bytes"] = srv.peak_used
        m["throughput_ratio_busy"] = m["cell_steps_per_s"] / max(1e-300, alone["cell_steps_per_s"])
        m["throughput_ratio_wall"] = (m["cell_steps_per_s_wall"]
                                      / max(1e-300, alone["cell_steps_per_s"]))
        m["p50_ratio_vs_alone"] = m["p50_step_ms"] / max(1e-300, alone["p50_step_ms"])
        m["p99_ratio_vs_alone"] = m["p99_step_ms"] / max(1e-300, alone["p99_step_ms"])
        out[key] = m
        del srv
    return out


def profile_step(argv=None):
    """``python bench.py --profile-step [options]``: one model step inside an
    NVTX range "step", for profilers.

    Builds the decaying-turbulence workload on an n x n periodic grid, sets
    psi, the diagnostics and dt (CFL 0.8), runs one warm-up step, then K steps
    inside the range (eager launches, so a profiler sees every kernel with
    its own grid) and prints the coarse level, the coarse operator's size and
    the solver statistics.  With ncu, ``--nvtx --nvtx-include "step/"`` keeps
    only the launches of the profiled steps.  ``--ensemble N`` profiles the
    batched step of the N-instance ensemble of ``workloads.ensemble(N,
    seed=4)`` instead (G groups of batched launches, merge policy P; G = 0:
    every instance's own graph on streams; coarse switch D levels below each
    instance's first allowed level)."""
    ap = argparse.ArgumentParser(prog="bench.py --profile-step")
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--precision", default="fp64", choices=("fp64", "mixed"))
    ap.add_argument("--coarse-level", type=int, default=None)
    ap.add_argument("--no-coarse-operator", action="store_true")
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--ensemble", type=int, default=0)
    ap.add_argument("--groups", type=int, default=1)
    ap.add_argument("--policy", type=int, default=1)
    ap.add_argument("--coarse-offset", type=int, default=0)
    ap.add_argument("--balanced", action="store_true")
    a = ap.parse_args(argv)
    import torch
    from fluid2d_gb300 import engine, workloads
    if a.ensemble > 0:
        E = engine.ensemble_from_workloads(workloads.ensemble(a.ensemble, seed=4),
                                           precision=a.precision, batched=a.groups > 0,
                                           groups=max(1, a.groups), policy=a.policy)
        if a.balanced and E.batch is not None:
            E.build_batch(max(1, a.groups), a.policy, balanced=True)
        if a.coarse_offset:
            E.coarse_offset(a.coarse_offset)
        E.run(1)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("step")
        E.run(a.steps)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        if E.batch is not None:
            print("batched launches per step %d, recorded operations %d" % E.batch_info())
        return
    M = engine.from_workload(workloads.turbulence(a.n, a.n), precision=a.precision, dt=1e-3)
    if a.coarse_level is not None:
        M.coarse_switch(a.coarse_level)
    if a.no_coarse_operator:
        M.coarse_operator(False)
    M.set_psi_from_vorticity()
    d = M.diagnostics()
    M.set_dt(0.8 * M.dx / d["maxspeed"])
    M.run(1)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("step")
    M.run(a.steps)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print("coarse level %d of %d, coarse operator %d points, solve %s"
          % (M.coarse_level, M.nlevs, M.coarse_operator(), M.solve_stats()))


def main():
    if "--profile-step" in sys.argv[1:]:
        profile_step([x for x in sys.argv[1:] if x != "--profile-step"])
        return
    a = parse()
    rank, world, local = dist_info()
    if a.impl == "reference":
        run_reference(a, rank, world)
        return
    run_ours(a, rank, world, local)


if __name__ == "__main__":
    main()
