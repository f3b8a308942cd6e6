"""Host logic of the serving loop (no GPU): admission against the HBM
budget, continuous batching (requests join and leave between ticks), FIFO
order, retirement freeing memory, rejection of what can never fit."""
import numpy as np

from fluid2d_gb300 import serve, workloads as W


class FakeModel(object):
    def __init__(self, wl, precision):
        self.wl = wl
        self.steps = 0

    def nbytes(self):
        return serve.estimate_bytes(self.wl, "fp64")

    def status(self):
        # a request whose workload says so fails after that many steps
        fail = self.wl.get("fail_after")
        return 2 if fail is not None and self.steps >= fail else 0


def fake_step(models):
    for m in models:
        m.steps += 1
    return 1e-3 * len(models)


def wl(n):
    return {"nx": n, "ny": n, "model": "euler"}


def test_admission_respects_the_budget_and_fifo():
    budget = serve.estimate_bytes(wl(256), "fp64") * 2 + 1
    s = serve.Server(budget, precision="fp64", make_model=FakeModel, step_models=fake_step)
    reqs = [serve.Request(k, 0., wl(256), 3) for k in range(5)]
    for r in reqs:
        s.submit(r)
    s.admit(0.)
    assert [r.rid for r in s.active] == [0, 1]
    assert s.used <= budget
    s.tick(0.)
    s.tick(0.)
    s.tick(0.)  # 0 and 1 finish, memory freed
    assert [r.rid for r in s.finished] == [0, 1]
    s.admit(0.)
    assert [r.rid for r in s.active] == [2, 3]


def test_continuous_batching_requests_join_and_leave():
    budget = serve.estimate_bytes(wl(128), "fp64") * 3 + 1
    s = serve.Server(budget, precision="fp64", make_model=FakeModel, step_models=fake_step)
    s.submit(serve.Request(0, 0., wl(128), 1))
    s.submit(serve.Request(1, 0., wl(128), 4))
    s.admit(0.)
    s.tick(0.)                     # request 0 leaves after one step
    s.submit(serve.Request(2, 0., wl(128), 2))
    s.admit(0.)                    # request 2 joins while 1 is running
    assert sorted(r.rid for r in s.active) == [1, 2]
    while s.active:
        s.tick(0.)
    assert sorted(r.rid for r in s.finished) == [0, 1, 2]
    assert all(len(r.latencies) == r.steps for r in s.finished)


def test_too_large_requests_are_rejected():
    s = serve.Server(1000, make_model=FakeModel, step_models=fake_step)
    assert not s.submit(serve.Request(0, 0., wl(512), 1))
    assert len(s.rejected) == 1


def test_run_and_metrics_with_fakes():
    stream = [(0.001 * k, wl(128), 2 + k % 3) for k in range(10)]
    budget = serve.estimate_bytes(wl(128), "fp64") * 4
    s = serve.Server(budget, precision="fp64", make_model=FakeModel, step_models=fake_step)
    m = s.run(stream, time_scale=100.)
    assert m["requests"] == 10 and m["rejected"] == 0
    assert m["cell_steps"] == sum(128 * 128 * st for _, _, st in stream)
    assert m["p99_step_ms"] >= m["p50_step_ms"] > 0


def test_served_stream_generator():
    st = W.served_stream(count=20, seed=5, side_min=128, side_max=512)
    ts = [t for t, _, _ in st]
    assert ts == sorted(ts)
    kinds = {w["model"] for _, w, _ in st}
    assert kinds <= {"euler", "boussinesq"}
    for _, w, steps in st:
        assert w["nx"] % 128 == 0 and w["ny"] % 128 == 0
        assert 50 <= steps <= 500
        assert w["msk"].shape == (w["ny"] + 6, w["nx"] + 6)
        assert abs(w["Lx"] / w["nx"] - w["Ly"] / w["ny"]) < 1e-15


def test_bogus_requests_are_rejected_with_their_reason():
    s = serve.Server(1 << 40, precision="fp64", make_model=FakeModel, step_models=fake_step)
    bad = [serve.Request(0, 0., {"nx": 0, "ny": 64, "model": "euler"}, 3),
           serve.Request(1, 0., {"nx": 64, "ny": 64.5, "model": "euler"}, 3),
           serve.Request(2, 0., {"nx": 64, "ny": 64, "model": "sqg"}, 3),
           serve.Request(3, 0., {"nx": 64, "ny": 64, "model": "euler",
                                 "msk": np.ones((10, 10), np.int8)}, 3),
           serve.Request(4, 0., wl(64), 0)]
    for r in bad:
        assert not s.submit(r)
    assert [r.rid for r in s.rejected] == [0, 1, 2, 3, 4]
    assert all(r.error for r in s.rejected)
    assert not s.queue


def test_a_request_the_engine_refuses_fails_alone():
    def make(w, precision):
        if w.get("refuse"):
            raise RuntimeError("f2d_model_create failed")
        return FakeModel(w, precision)
    s = serve.Server(1 << 40, precision="fp64", make_model=make, step_models=fake_step)
    s.submit(serve.Request(0, 0., dict(wl(64), refuse=True), 2))
    s.submit(serve.Request(1, 0., wl(64), 2))
    s.admit(0.)
    assert [r.rid for r in s.active] == [1]
    assert s.rejected[0].rid == 0 and "set-up failed" in s.rejected[0].error
    while s.active:
        s.tick(0.)
    assert [r.rid for r in s.finished] == [1]


def test_a_failing_simulation_is_retired_alone():
    budget = serve.estimate_bytes(wl(128), "fp64") * 3 + 1
    s = serve.Server(budget, precision="fp64", make_model=FakeModel, step_models=fake_step)
    s.submit(serve.Request(0, 0., wl(128), 5))
    s.submit(serve.Request(1, 0., dict(wl(128), fail_after=2), 5))
    s.submit(serve.Request(2, 0., wl(128), 5))
    s.admit(0.)
    used = s.used
    s.tick(0.)
    assert len(s.active) == 3
    s.tick(0.)  # request 1 reports a blow-up after its second step
    assert [r.rid for r in s.active] == [0, 2]
    assert [r.rid for r in s.failed] == [1]
    assert "blow-up" in s.failed[0].error and s.failed[0].model is None
    assert s.used < used  # its memory is freed
    while s.active:
        s.tick(0.)
    assert [r.rid for r in s.finished] == [0, 2]
    assert all(r.done == 5 for r in s.finished)
    m = serve.metrics(s.finished, 1., 1., s.rejected, s.failed)
    assert m["failed"] == 1 and m["requests"] == 2


def test_admission_uses_measured_sizes():
    class Big(FakeModel):
        def nbytes(self):
            return 3 * serve.estimate_bytes(self.wl, "fp64")
    budget = serve.estimate_bytes(wl(128), "fp64") * 4
    s = serve.Server(budget, precision="fp64", make_model=Big, step_models=fake_step)
    for k in range(3):
        s.submit(serve.Request(k, 0., wl(128), 2))
    s.admit(0.)
    # the first model measured 3x the estimate: the second no longer fits
    assert [r.rid for r in s.active] == [0]
    assert s.used <= budget
    assert s.per_point["euler"] > serve.BYTES_PER_POINT["fp64"]
    assert [r.rid for r in s.queue] == [1, 2]
    while s.active or s.queue:
        s.admit(0.)
        s.tick(0.)
    assert [r.rid for r in s.finished] == [0, 1, 2]


class FakeChunks(object):
    """Free-running chunks on the host: a chunk of n steps finishes at the
    next poll, after n ms; the model counts its steps."""

    def launch(self, r, n):
        r.inflight = n
        r.model.steps += n

    def poll(self, r):
        return 1e-3 * r.inflight

    def wait(self):
        pass


def test_free_running_serving_admits_retires_and_isolates():
    budget = serve.estimate_bytes(wl(128), "fp64") * 2 + 1
    s = serve.Server(budget, precision="fp64", make_model=FakeModel, chunks=FakeChunks(),
                     max_active=2)
    stream = [(0., wl(128), 20), (0., dict(wl(128), fail_after=5), 20), (0., wl(128), 7),
              (0., {"nx": 3, "ny": 64, "model": "euler"}, 5)]
    m = s.run_free(stream, chunk=4, time_scale=100.)
    assert m["requests"] == 2 and m["failed"] == 1 and m["rejected"] == 1
    assert sorted(r.rid for r in s.finished) == [0, 2]
    assert s.failed[0].rid == 1 and "blow-up" in s.failed[0].error
    assert all(len(r.latencies) == r.steps for r in s.finished)
    assert all(abs(x - 1e-3) < 1e-12 for r in s.finished for x in r.latencies)
    assert s.used == 0
