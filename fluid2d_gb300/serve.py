"""Serving loop: simulations arrive as requests and are stepped together.

A request is (model, grid, mask, initial fields, step count).  The server
keeps a FIFO of arrived requests and admits the head whenever its estimated
device memory fits in the HBM budget beside the running ones; every admitted
simulation keeps its state resident on the GPU.  Each tick advances every
running simulation by one step -- its captured step graph replayed on one of
`nstreams` CUDA streams, so the kernels of different simulations overlap --
and retires the ones that have done all their steps, which frees memory for
the next admissions (continuous batching: requests join and leave between
ticks).  Per-step latency of a request is the duration of the tick that
advanced it.

`run_one_at_a_time` is the comparator: the same requests, one after the
other, each alone on the GPU.
"""
import time

import numpy as np

# device bytes per grid point (halo included) of a model and its multigrid
# hierarchy, measured from the engine's allocations, with a margin
BYTES_PER_POINT = {"fp64": 560., "mixed": 760.}


def estimate_bytes(wl, precision):
    pts = (wl["nx"] + 6) * (wl["ny"] + 6)
    return int(BYTES_PER_POINT[precision] * pts) + (4 << 20)


class Request(object):
    def __init__(self, rid, arrival, wl, steps):
        self.rid = rid
        self.arrival = arrival
        self.wl = wl
        self.steps = steps
        self.done = 0
        self.model = None
        self.nbytes = 0
        self.admitted = None
        self.finished = None
        self.latencies = []

    @property
    def cells(self):
        return self.wl["nx"] * self.wl["ny"]


class Server(object):
    """Continuous-batching server over an HBM budget.

    `make_model(wl, precision)` builds an initialised model; `step_models`
    advances a list of models by one step and returns the tick's duration in
    seconds.  Both default to the GPU engine; tests may pass host fakes.
    """

    def __init__(self, hbm_budget, precision="mixed", nstreams=32, make_model=None,
                 step_models=None, max_active=None, clock=time.perf_counter, on_finish=None):
        self.budget = int(hbm_budget)
        self.precision = precision
        self.nstreams = nstreams
        self.make_model = make_model or _gpu_make_model
        self.step_models = step_models or _GpuStepper(nstreams).step
        self.max_active = max_active
        self.clock = clock
        self.on_finish = on_finish
        self.used = 0
        self.queue = []
        self.active = []
        self.finished = []
        self.rejected = []
        self.ticks = []

    def submit(self, req):
        if estimate_bytes(req.wl, self.precision) > self.budget:
            self.rejected.append(req)  # can never fit
            return False
        self.queue.append(req)
        return True

    def admit(self, now):
        while self.queue:
            if self.max_active is not None and len(self.active) >= self.max_active:
                break
            req = self.queue[0]
            need = estimate_bytes(req.wl, self.precision)
            if self.used + need > self.budget:
                break
            self.queue.pop(0)
            req.model = self.make_model(req.wl, self.precision)
            req.nbytes = max(need, _model_bytes(req.model))
            self.used += req.nbytes
            req.admitted = now
            self.active.append(req)

    def tick(self, now):
        if not self.active:
            return 0.
        dt = self.step_models([r.model for r in self.active])
        self.ticks.append((now, len(self.active), sum(r.cells for r in self.active), dt))
        keep = []
        for r in self.active:
            r.done += 1
            r.latencies.append(dt)
            if r.done >= r.steps:
                r.finished = now + dt
                if self.on_finish is not None:
                    self.on_finish(r)
                self.used -= r.nbytes
                r.model = None  # frees the device memory
                self.finished.append(r)
            else:
                keep.append(r)
        self.active = keep
        return dt

    def run(self, stream, time_scale=1.0):
        """Serve (arrival, wl, steps) tuples; arrival times are honoured in
        wall-clock time divided by `time_scale`.  Returns the metrics."""
        reqs = [Request(k, t, wl, st) for k, (t, wl, st) in enumerate(stream)]
        t0 = self.clock()
        nxt = 0
        busy = 0.
        while nxt < len(reqs) or self.queue or self.active:
            now = (self.clock() - t0) * time_scale
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                self.submit(reqs[nxt])
                nxt += 1
            self.admit(now)
            if self.active:
                busy += self.tick(now)
            elif nxt < len(reqs):
                wait = (reqs[nxt].arrival - now) / time_scale
                if wait > 0:
                    time.sleep(min(wait, 0.05))
            elif self.queue and not self.active:
                # head cannot be admitted even with nothing running
                self.rejected.append(self.queue.pop(0))
        wall = self.clock() - t0
        return metrics(self.finished, wall, busy, self.rejected)


def metrics(finished, wall, busy, rejected=()):
    lat = np.array([x for r in finished for x in r.latencies]) if finished else np.zeros(1)
    cell_steps = float(sum(r.cells * r.steps for r in finished))
    return {"requests": len(finished), "rejected": len(rejected), "cell_steps": cell_steps,
            "wall_s": wall, "busy_s": busy,
            "cell_steps_per_s": cell_steps / busy if busy > 0 else 0.,
            "cell_steps_per_s_wall": cell_steps / wall if wall > 0 else 0.,
            "p50_step_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_step_ms": float(np.percentile(lat, 99) * 1e3)}


def _model_bytes(m):
    try:
        return int(m.nbytes())
    except Exception:
        return 0


def _gpu_make_model(wl, precision):
    from . import engine
    m = engine.from_workload(wl, precision=precision)
    m.set_psi_from_vorticity()
    d = m.diagnostics()
    if d["maxspeed"] > 0:
        m.set_dt(0.8 * min(m.dx, m.dy) / d["maxspeed"])
    return m


class _GpuStepper(object):
    def __init__(self, nstreams):
        import torch
        self.torch = torch
        self.streams = [torch.cuda.Stream() for _ in range(max(1, nstreams))]

    def step(self, models):
        torch = self.torch
        cur = torch.cuda.current_stream()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(cur)
        for s in self.streams:
            s.wait_stream(cur)
        for i, m in enumerate(models):
            with torch.cuda.stream(self.streams[i % len(self.streams)]):
                m.run(1, graph=True)
        for s in self.streams:
            cur.wait_stream(s)
        e1.record(cur)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3


def run_one_at_a_time(stream, precision="fp64", make_model=None):
    """The comparator: every request alone on the GPU, in arrival order;
    per-step latency is that request's own step time."""
    import torch
    make_model = make_model or _gpu_make_model
    fin = []
    busy = 0.
    t0 = time.perf_counter()
    s = torch.cuda.Stream()
    for k, (t, wl, steps) in enumerate(stream):
        r = Request(k, t, wl, steps)
        m = make_model(wl, precision)
        with torch.cuda.stream(s):
            m.run(1, graph=True)  # capture
            s.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            m.run(steps - 1, graph=True)
            e1.record(s)
            e1.synchronize()
        ms = e0.elapsed_time(e1) / max(1, steps - 1)
        r.latencies = [ms * 1e-3] * steps
        r.done = steps
        busy += ms * 1e-3 * steps
        fin.append(r)
        del m
    return metrics(fin, time.perf_counter() - t0, busy)
