"""Serving loop: simulations arrive as requests and are stepped together.

A request is (model, grid, mask, initial fields, step count).  The server
keeps a FIFO of arrived requests and admits the head whenever its device
memory fits in the HBM budget beside the running ones -- estimated from the
bytes per grid point measured on the models already built (nbytes()), and
checked against the built model's own nbytes() before it runs; every
admitted simulation keeps its state resident on the GPU.  A request the
engine cannot serve (unknown model, bad grid, too large) is rejected with
its reason; a simulation whose run fails (non-finite values, blow-up,
diverged solve: the model's device status word, read after every tick) is
retired alone with its reason, and the others go on unchanged.  Each tick advances every
running simulation by one step -- its captured step graph replayed on one of
`nstreams` CUDA streams, so the kernels of different simulations overlap --
and retires the ones that have done all their steps, which frees memory for
the next admissions (continuous batching: requests join and leave between
ticks).  Per-step latency of a request is the duration of the tick that
advanced it.

`run_free` serves the same stream with every admitted simulation running free
on its own stream (chunks of steps queued as the previous chunk finishes)
instead of in lockstep ticks.

`run_one_at_a_time` is the comparator: the same requests, one after the
other, each alone on the GPU.
"""
import time

import numpy as np

# device bytes per grid point (halo included) of a model and its multigrid
# hierarchy, with a margin: the first estimate for a (model, precision) whose
# size the server has not measured yet; afterwards the largest measured
# nbytes()/point of that kind is used
BYTES_PER_POINT = {"fp64": 560., "mixed": 760.}
MODELS = ("euler", "boussinesq", "quasigeostrophic")


def estimate_bytes(wl, precision, per_point=None):
    pts = (wl["nx"] + 6) * (wl["ny"] + 6)
    return int((per_point or BYTES_PER_POINT[precision]) * pts) + (4 << 20)


def check_request(wl, steps):
    """Why a request cannot be served (None if it can): unknown model, grid
    sides that are not integers in [4, 32768], a mask of the wrong shape, a
    step count below 1."""
    if wl.get("model") not in MODELS:
        return "unknown model %r" % (wl.get("model"),)
    nx, ny = wl.get("nx"), wl.get("ny")
    if not all(isinstance(v, (int, np.integer)) and 4 <= v <= 32768 for v in (nx, ny)):
        return "bad grid size %r x %r" % (nx, ny)
    msk = wl.get("msk")
    if msk is not None and tuple(np.shape(msk)) != (ny + 6, nx + 6):
        return "mask shape %s is not (ny+6, nx+6)" % (np.shape(msk),)
    if not (isinstance(steps, (int, np.integer)) and steps >= 1):
        return "bad step count %r" % (steps,)
    return None


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
        self.error = None  # why it was rejected or retired early

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
                 step_models=None, max_active=None, clock=time.perf_counter, on_finish=None,
                 chunks=None):
        self.budget = int(hbm_budget)
        self.precision = precision
        self.nstreams = nstreams
        self.make_model = make_model or _gpu_make_model
        self._step_models = step_models
        self._chunks = chunks
        self.read_status = _read_status
        self.max_active = max_active
        self.clock = clock
        self.on_finish = on_finish
        self.used = 0
        self.queue = []
        self.active = []
        self.finished = []
        self.rejected = []
        self.failed = []
        self.ticks = []
        self.peak_used = 0    # the most device memory admitted at once
        self.peak_active = 0  # the most simulations running at once
        self.per_point = {}  # measured device bytes per grid point, per model

    def step_models(self, models):
        if self._step_models is None:
            self._step_models = _GpuStepper(self.nstreams).step
        return self._step_models(models)

    @property
    def chunks(self):
        if self._chunks is None:
            self._chunks = _GpuChunks(self.nstreams)
        return self._chunks

    def _estimate(self, wl):
        return estimate_bytes(wl, self.precision, self.per_point.get(wl["model"]))

    def _reject(self, req, why):
        req.error = why
        self.rejected.append(req)
        return False

    def submit(self, req):
        why = check_request(req.wl, req.steps)
        if why:
            return self._reject(req, why)
        if self._estimate(req.wl) > self.budget:
            return self._reject(req, "needs more than the HBM budget")  # can never fit
        self.queue.append(req)
        return True

    def admit(self, now):
        while self.queue:
            if self.max_active is not None and len(self.active) >= self.max_active:
                break
            req = self.queue[0]
            need = self._estimate(req.wl)
            if self.used + need > self.budget:
                break
            self.queue.pop(0)
            try:
                req.model = self.make_model(req.wl, self.precision)
            except Exception as exc:  # a request the engine refuses fails alone
                self._reject(req, "model set-up failed: %s" % exc)
                continue
            got = _model_bytes(req.model)
            if got:
                # admission on measured sizes: the largest bytes per point seen
                pp = (got - (4 << 20)) / float((req.wl["nx"] + 6) * (req.wl["ny"] + 6))
                kind = req.wl["model"]
                self.per_point[kind] = max(self.per_point.get(kind, 0.), pp)
            req.nbytes = got or need
            if self.used + req.nbytes > self.budget:
                # larger than estimated: back to the head of the queue until
                # memory frees up
                req.model = None
                self.queue.insert(0, req)
                break
            self.used += req.nbytes
            req.admitted = now
            self.active.append(req)
            self.peak_used = max(self.peak_used, self.used)
            self.peak_active = max(self.peak_active, len(self.active))

    def tick(self, now):
        if not self.active:
            return 0.
        dt = self.step_models([r.model for r in self.active])
        self.ticks.append((now, len(self.active), sum(r.cells for r in self.active), dt))
        keep = []
        status = self.read_status([r.model for r in self.active])
        for r, bits in zip(self.active, status):
            r.done += 1
            r.latencies.append(dt)
            if bits:
                # this instance alone leaves: the others share nothing with it
                r.error = "retired after step %d: %s" % (r.done, _status_text(bits))
                self._release(r, now + dt)
                self.failed.append(r)
            elif r.done >= r.steps:
                if self.on_finish is not None:
                    self.on_finish(r)
                self._release(r, now + dt)
                self.finished.append(r)
            else:
                keep.append(r)
        self.active = keep
        return dt

    def _release(self, r, when):
        r.finished = when
        self.used -= r.nbytes
        r.model = None  # frees the device memory

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
                self._reject(self.queue.pop(0), "does not fit the HBM budget alone")
        wall = self.clock() - t0
        return metrics(self.finished, wall, busy, self.rejected, self.failed)


    def run_free(self, stream, chunk=8, time_scale=1.0):
        """Serve (arrival, wl, steps) tuples with every admitted simulation
        running free on its own CUDA stream: `chunk` steps (its captured step
        graph replayed) are queued at a time, and the next chunk as soon as
        the last one has finished, so a small simulation is not held back by
        a large one as in the lockstep ticks of run(); the per-step latency of
        a step is its chunk's duration on the device over the chunk's steps.
        Admission, retirement, failure isolation (status words read after
        each chunk) and the budget are those of run().  Returns the metrics."""
        reqs = [Request(k, t, wl, st) for k, (t, wl, st) in enumerate(stream)]
        t0 = self.clock()
        nxt = 0
        busy = 0.
        last = t0
        while nxt < len(reqs) or self.queue or self.active:
            tnow = self.clock()
            if self.active:
                busy += tnow - last
            last = tnow
            now = (tnow - t0) * time_scale
            while nxt < len(reqs) and reqs[nxt].arrival <= now:
                self.submit(reqs[nxt])
                nxt += 1
            before = len(self.active)
            self.admit(now)
            for r in self.active[before:]:
                self.chunks.launch(r, min(chunk, r.steps - r.done))
            # chunks that have finished: account, check, go on or retire
            done = [(r, self.chunks.poll(r)) for r in self.active]
            done = [(r, sec) for r, sec in done if sec is not None]
            if done:
                status = self.read_status([r.model for r, _ in done])
                gone = set()
                for (r, sec), bits in zip(done, status):
                    n = r.inflight
                    r.done += n
                    r.latencies.extend([sec / n] * n)
                    if bits:
                        r.error = "retired after step %d: %s" % (r.done, _status_text(bits))
                        self._release(r, now)
                        self.failed.append(r)
                        gone.add(id(r))
                    elif r.done >= r.steps:
                        if self.on_finish is not None:
                            self.on_finish(r)
                        self._release(r, now)
                        self.finished.append(r)
                        gone.add(id(r))
                    else:
                        self.chunks.launch(r, min(chunk, r.steps - r.done))
                self.active = [r for r in self.active if id(r) not in gone]
            elif not self.active:
                if nxt < len(reqs):
                    wait = (reqs[nxt].arrival - now) / time_scale
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                elif self.queue:
                    self._reject(self.queue.pop(0), "does not fit the HBM budget alone")
            else:
                self.chunks.wait()
        wall = self.clock() - t0
        return metrics(self.finished, wall, busy, self.rejected, self.failed)


def metrics(finished, wall, busy, rejected=(), failed=()):
    lat = np.array([x for r in finished for x in r.latencies]) if finished else np.zeros(1)
    cell_steps = float(sum(r.cells * r.steps for r in finished))
    return {"requests": len(finished), "rejected": len(rejected), "failed": len(failed),
            "cell_steps": cell_steps,
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


def _read_status(models):
    """Status words of the models (0 = healthy): engine models in one
    synchronisation, others (host fakes) through their own status()."""
    from . import engine
    if models and all(isinstance(m, engine.Model) for m in models):
        return engine.statuses(models)
    return [int(m.status()) if hasattr(m, "status") else 0 for m in models]


def _status_text(bits):
    from .engine import status_text
    return status_text(bits)


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


class _GpuChunks(object):
    """Chunks of steps of each request on its own stream (free-running
    serving): launch() queues a chunk bracketed by CUDA events, poll() gives
    its device duration in seconds once it has finished, else None."""

    def __init__(self, nstreams):
        import torch
        self.torch = torch
        self.streams = [torch.cuda.Stream() for _ in range(max(1, nstreams))]
        self.next = 0

    def launch(self, r, n):
        torch = self.torch
        if getattr(r, "stream", None) is None:
            r.stream = self.streams[self.next % len(self.streams)]
            self.next += 1
            r.ev0 = torch.cuda.Event(enable_timing=True)
            r.ev1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(r.stream):
            r.ev0.record(r.stream)
            r.model.run(n, graph=True)
            r.ev1.record(r.stream)
        r.inflight = n

    def poll(self, r):
        if not r.ev1.query():
            return None
        return r.ev0.elapsed_time(r.ev1) * 1e-3

    def wait(self):
        time.sleep(50e-6)


def run_one_at_a_time(stream, precision="fp64", make_model=None, timed_steps=None):
    """The comparator: every request alone on the GPU, in arrival order;
    per-step latency is that request's own step time.  With `timed_steps`,
    each request is timed over that many steps after its graph capture and
    its time is its step count times the mean (a fixed-dt step costs the same
    every step); otherwise every step runs."""
    import torch
    make_model = make_model or _gpu_make_model
    fin = []
    busy = 0.
    t0 = time.perf_counter()
    s = torch.cuda.Stream()
    for k, (t, wl, steps) in enumerate(stream):
        r = Request(k, t, wl, steps)
        m = make_model(wl, precision)
        n = steps - 1 if timed_steps is None else max(1, min(steps - 1, int(timed_steps)))
        with torch.cuda.stream(s):
            m.run(1, graph=True)  # capture
            s.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            m.run(n, graph=True)
            e1.record(s)
            e1.synchronize()
        ms = e0.elapsed_time(e1) / max(1, n)
        r.latencies = [ms * 1e-3] * steps
        r.done = steps
        busy += ms * 1e-3 * steps
        fin.append(r)
        del m
    out = metrics(fin, time.perf_counter() - t0, busy)
    if timed_steps is not None:
        out["steps_timed_per_request"] = int(timed_steps)
    return out
