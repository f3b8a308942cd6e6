#!/usr/bin/env python
"""Throughput of the Fluid2d time step on GB300: cell-steps/s per RK3 step.

Workload (the headline configuration): Euler 2D decaying turbulence on a
doubly periodic 1024 x 1024 unit box, random-phase vorticity with
E(k) ~ k^3 exp(-(k/10)^2), rms 1 (seeded synthetic data: the reference
publishes no dataset), 5th-order upwind advection, RK3-SSP, multigrid
Poisson inversion (two V-cycles per inverting stage, full F-cycle solve after
every step), float64, fixed dt from CFL 0.8 on the initial max|u|.

One bench "step" is one iteration of the reference's time loop
(core/fluid2d.py:237-268): set_dt, model.step (3 RK stages + solve),
diagnostics.  value = interior cells x steps / device time.  The working set
(state, RK tendencies, stage states, multigrid hierarchy, ~0.3 GB) is larger
than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=NX, help="grid side (default 1024)")
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ensemble-steps", type=int, default=20)
    ap.add_argument("--served-requests", type=int, default=24)
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the ensemble and served-stream measurements")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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
def _cpu_worker(args):
    """Step the oracle (the reference's CPU path restated) for a time budget."""
    n, budget, seed = args
    sys.path.insert(0, ROOT)
    from fluid2d_gb300 import workloads as W
    from oracle import stepper
    wl = W.turbulence(n, n, seed=2)
    p, M = stepper.from_workload(wl)
    dt = 0.8 * min(M.grid.dx, M.grid.dy) / M.diags["maxspeed"]
    t0 = time.perf_counter()
    steps = 0
    t = 0.
    while True:
        t = stepper.run(M, p, 1, dt, t=t)
        steps += 1
        if time.perf_counter() - t0 >= budget:
            break
    return steps, time.perf_counter() - t0


# float64 FMA throughput of a GB300 of this machine (independent DFMA chains on
# every SM, CUDA events), used only if the live measurement (f2d_fp64_peak)
# fails: the FP64-ALU roofline of the float64 kernels
FP64_PEAK_TFLOPS = 1.20
SMOOTH_DRAM_BYTES_PER_POINT = (20111360 + 0 + 20073472 + 0) / 1060900.


def cpu_baseline(n, budget, cores):
    """Cell-steps/s of the oracle path on `cores` host processes."""
    from oracle import oracle
    oracle.build()
    if cores == 1:
        steps, wall = _cpu_worker((n, budget, 0))
        return n * n * steps / wall, "1 process, %d steps of the %dx%d workload in %.1f s" % (
            steps, n, n, wall)
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(n, budget, k) for k in range(cores)])
    wall = time.perf_counter() - t0
    total = sum(s for s, _ in res)
    slowest = max(w for _, w in res)
    return n * n * total / slowest, (
        "%d processes, each stepping its own %dx%d copy for ~%.0f s (%d steps in total)"
        % (cores, n, n, budget, total))


def run_reference(a, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    K, W = a.steps, a.warmup
    # the whole --steps/--warmup run is one bounded sample per core
    val, sample = cpu_baseline(a.n, a.cpu_sample_s, cores)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT,
            "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": "euler-decaying-turbulence-%dx%d-perio-fp64"
                                            % (a.n, a.n), "nx": a.n, "ny": a.n},
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
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
    ms = e0.elapsed_time(e1)
    if world > 1:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    ms_step = ms / a.steps
    value = world * n * n * a.steps / (ms * 1e-3)
    nite, res, st = M.solve_stats()
    diags = M.read_diags()

    # ---- the mixed form on the same workload (FP32 fluxes and multigrid
    # cycles inside an FP64 defect correction; FP64 state, RK and diagnostics)
    mixed = None
    try:
        mixed = bench_mixed(engine, wl, dt, s0, a, stream, world)
    except Exception as exc:
        print("mixed form failed: %s" % exc, file=sys.stderr)

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
    pts = (n + 6) * (n + 6)
    # one smoothtwicewitha call reads x, b, msk and writes x: 8+8+1+8 = 25 B/point
    alg_bytes = 25 * pts
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg_bytes / (probe_ms * 1e-3) / 1e9 if probe_ms > 0 else None
    # dram__bytes_read.sum + dram__bytes_write.sum of one smoothtwicewitha call
    # (k_sweep1 + k_sweep2) per grid point, from the ncu capture summarised in
    # profiles/k_sweep_turbulence_1024_fp64_dram.md (1024^2, 1060900 points)
    traffic = SMOOTH_DRAM_BYTES_PER_POINT * pts
    # the same kernel against the float64 pipe, its real bound on this part:
    # one damped-Jacobi update is 1 mul + 7 fma + 1 sub + 1 mul + 1 fma =
    # 19 flops, two sweeps per call
    fp64_flops = 2 * 19 * pts
    fp64_achieved = fp64_flops / (probe_ms * 1e-3) / 1e12 if probe_ms > 0 else None
    fp64_peak, fp64_src = FP64_PEAK_TFLOPS, "earlier FMA-chain measurement on this pool"
    try:
        import ctypes as _ct
        from fluid2d_gb300 import _lib as _l
        _v = _ct.c_double()
        if _l.lib().f2d_fp64_peak(_ct.byref(_v)) == 0 and _v.value > 0:
            fp64_peak, fp64_src = _v.value, "f2d_fp64_peak: FMA chains measured live on this GPU"
    except Exception as exc:
        print("fp64 peak failed: %s" % exc, file=sys.stderr)

    # ---- e2e through the public API with host buffers: every step uploads
    # the state (Var.state) from pinned memory, steps, reads it back
    state_host = torch.empty(M.var.state.shape, dtype=torch.float64).pin_memory()
    state_host.copy_(M.var.state.cpu())
    h2d = d2h = state_host.numel() * 8
    with torch.cuda.stream(stream):
        for _ in range(2):
            M.var.state.copy_(state_host, non_blocking=True)
            M.run(1, graph=True)
            state_host.copy_(M.var.state, non_blocking=True)
        stream.synchronize()
        barrier()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(a.e2e_steps):
            M.var.state.copy_(state_host, non_blocking=True)
            M.run(1, graph=True)
            state_host.copy_(M.var.state, non_blocking=True)
        f1.record(stream)
        f1.synchronize()
    e2e_ms = f0.elapsed_time(f1)
    if world > 1:
        t = torch.tensor([e2e_ms], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e_val = world * n * n * a.e2e_steps / (e2e_ms * 1e-3)

    extra = {}
    # the ensemble and the served stream tune their own launch structure;
    # the level kernels go back to their default tiles and block sizes
    try:
        from fluid2d_gb300 import _lib as _l
        _l.lib().f2d_set_level_tiles(0)
        _l.lib().f2d_set_level_threads(0)
    except Exception as exc:
        print("level tiles reset failed: %s" % exc, file=sys.stderr)
    if not a.no_extra and rank == 0:
        for key, fn in (("ensemble", bench_ensemble), ("served", bench_served)):
            try:
                extra[key] = fn(a)
            except Exception as exc:
                print("%s failed: %s" % (key, exc), file=sys.stderr)
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return
    cpu = None
    if not a.no_cpu_baseline:
        v, sample = cpu_baseline(n, a.cpu_sample_s, 1)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded random-phase vorticity, E(k)~k^3 exp(-(k/10)^2), rms 1",
        "config": {"workload": "euler-decaying-turbulence-%dx%d-perio-fp64" % (n, n),
                   "nx": n, "ny": n, "precision": "fp64", "cuda_graph": True,
                   "multigrid_levels": M.nlevs, "coarse_cta_from_level": M.coarse_level,
                   "coarse_operator_points": M.coarse_operator(),
                   "level_tiles": {"cta_target": tiles[0], "one_pass_threads": tiles[1]},
                   "solve_iterations_last_step": nite, "solve_residual_last_step": res,
                   "dt": dt, "maxspeed": diags.get("maxspeed"),
                   "l2": "working set > L2 (state, tendencies, hierarchy ~0.3 GB); no flush",
                   "parallelism": "replicas" if world > 1 else "single"},
        "roofline": {"kernel": "finest-level smoother (smoothtwicewitha: sweep1+sweep2)",
                     "bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                     "traffic": traffic, "launches_probed": nprobe,
                     "avg_launch_ms": probe_ms,
                     "alg_bytes_per_launch": alg_bytes,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback",
                     "fp64": {"achieved": fp64_achieved, "peak": fp64_peak,
                              "unit": "TFLOP/s",
                              "frac": (fp64_achieved / fp64_peak) if fp64_achieved else None,
                              "flops_per_launch": fp64_flops, "peak_source": fp64_src}},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "steps": a.e2e_steps},
        "mixed": mixed,
        "ensemble": extra.get("ensemble"),
        "served": extra.get("served"),
        "gpu_launches": kernels_per_step * a.steps,
        "clocks": clk.summary(),
        "libraries": [os.path.basename(so_path("product"))],
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def bench_mixed(engine, wl, dt, s0, a, stream, world):
    """Throughput of the mixed form, and its single-step error against the
    float64 path from the same state (per field, relative L2)."""
    import torch
    n = wl["nx"]
    Mm = engine.from_workload(wl, dt=dt, precision="mixed")
    Mm.var.state.copy_(s0)
    Mm.diagnostics()
    from fluid2d_gb300.autotune import tune_coarse_level
    tune_coarse_level(Mm, steps=3, warmup=1)
    Mm.var.state.copy_(s0)
    Mm.diagnostics()
    with torch.cuda.stream(stream):
        Mm.run(a.warmup, graph=True)
    stream.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        e0.record(stream)
        Mm.run(a.steps, graph=True)
        e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    nite, res, st = Mm.solve_stats()
    del Mm
    # one step of each form from the same (fresh) state
    A = engine.from_workload(wl, dt=dt)
    B = engine.from_workload(wl, dt=dt, precision="mixed")
    for M in (A, B):
        M.var.state.copy_(s0)
        M.diagnostics()
        M.run(1)
    torch.cuda.synchronize()
    err = {}
    for k, nm in enumerate(A.var.varname_list):
        ref = A.var.state[k]
        nrm = float(torch.linalg.vector_norm(ref))
        if nrm > 0:
            err[nm] = float(torch.linalg.vector_norm(B.var.state[k] - ref)) / nrm
    return {"value": world * n * n * a.steps / (ms * 1e-3), "unit": UNIT,
            "ms_per_step": ms / a.steps, "dtype": "f32 fluxes and multigrid, f64 defect "
            "correction, RK accumulation and diagnostics",
            "single_step_rel_l2_vs_f64": err, "solve_iterations_last_step": nite,
            "solve_residual_last_step": res}


def _structure(choice):
    off, groups, policy = choice
    lev = "coarse switch first+%d" % off
    if groups == 0:
        return "streams, " + lev
    return "batched groups=%d policy=%d, %s" % (groups, policy, lev)


def bench_ensemble(a):
    """Config: 96 independent Euler instances (sides log-uniform 64-768,
    multiples of 64, islands, 3-12 vortices; seed 4).  Batched = the launch
    structure the autotuner picks (fluid2d_gb300.autotune.tune_ensemble):
    groups of instances whose steps are merged into one launch per kernel,
    one graph per group on its own stream, or every instance's own step graph
    replayed on 32 streams; comparator = the plain float64 path, one instance
    at a time."""
    import torch
    from fluid2d_gb300 import engine, workloads as W
    from fluid2d_gb300.autotune import tune_ensemble
    wls = W.ensemble(96, seed=4)
    cells = sum(w["nx"] * w["ny"] for w in wls)
    out = {"instances": len(wls), "cells": cells, "steps": a.ensemble_steps}
    for prec in ("mixed", "fp64"):
        E = engine.ensemble_from_workloads(wls, precision=prec, nstreams=32)
        choice, times = tune_ensemble(E, steps=3, warmup=1)
        E.run(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        E.run(a.ensemble_steps)
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[prec + "_batched"] = {"cell_steps_per_s": cells * a.ensemble_steps / (ms * 1e-3),
                                  "ms_per_ensemble_step": ms / a.ensemble_steps,
                                  "launch_structure": _structure(choice),
                                  "tuning_ms_per_step": {_structure(k): round(v, 3)
                                                         for k, v in times.items()}}
        E.free_batch()
        del E
        torch.cuda.synchronize()
    # one at a time, plain float64
    tot_ms = 0.
    nst = max(2, a.ensemble_steps // 4)
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
    return out


def bench_served(a):
    """Config: served stream with Poisson arrivals at 40/s, 70 % Euler /
    30 % Boussinesq, sides 128-2048 (multiples of 128), HBM budget 150 GB.
    Bounded sample: the first --served-requests requests, step counts drawn
    from U[5, 50] (the full stream draws U[50, 500])."""
    from fluid2d_gb300 import serve, workloads as W
    stream = W.served_stream(count=a.served_requests, rate=40., seed=5, steps_min=5,
                             steps_max=50)
    srv = serve.Server(150e9, precision="mixed", nstreams=32)
    served = srv.run(stream)
    alone = serve.run_one_at_a_time(stream, precision="fp64")
    return {"sample": "%d requests, steps U[5,50], sides 128-2048, 70%% Euler / 30%% "
                      "Boussinesq, Poisson 40/s, budget 150 GB" % len(stream),
            "served_mixed_continuous_batching": served,
            "fp64_one_at_a_time": alone,
            "throughput_ratio": served["cell_steps_per_s"] / max(1e-300,
                                                                 alone["cell_steps_per_s"])}


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
