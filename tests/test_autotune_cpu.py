"""Host logic of fluid2d_gb300.autotune with fake models and fake timings (no
GPU): every candidate is timed, the fastest is kept set on the model or
ensemble, and choices are cached per (kind, grid, precision)."""
import contextlib
import types

import pytest

from fluid2d_gb300 import autotune


class _FakeStream(object):
    def wait_stream(self, other):
        pass

    def synchronize(self):
        pass


@pytest.fixture
def fake_cuda(monkeypatch):
    import torch
    monkeypatch.setattr(torch.cuda, "Stream", _FakeStream)
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a: _FakeStream())
    monkeypatch.setattr(torch.cuda, "stream", lambda s: contextlib.nullcontext())
    monkeypatch.setattr(autotune, "_cache", {})
    return torch


class FakeModel(object):
    """coarse_switch(level) as the engine's: sets the level, returns
    (current, first allowed, number of levels); run() steps at a cost that
    depends on the level."""

    def __init__(self, cost):
        self.cost = cost
        self.level = 6
        self.modelname = "euler"
        self.desc = types.SimpleNamespace(nx=1024, ny=1024, precision=0)

    def coarse_switch(self, level=None):
        if level is not None:
            self.level = level
        return self.level, 3, 9

    def run(self, n, graph=False):
        pass


def test_coarse_level_keeps_the_fastest_and_caches(fake_cuda, monkeypatch):
    cost = {3: 5.0, 4: 4.1, 5: 3.9, 6: 4.4, 7: 4.8, 8: 5.5, 9: 6.0}
    m = FakeModel(cost)
    monkeypatch.setattr(autotune, "_time", lambda run, steps, warmup: cost[m.level])
    best, times = autotune.tune_coarse_level(m)
    assert best == 5 and m.level == 5
    assert sorted(times) == list(range(3, 10))
    # cached: a second model of the same kind is set without timing
    m2 = FakeModel(cost)
    monkeypatch.setattr(autotune, "_time", lambda *a: pytest.fail("timed again"))
    assert autotune.tune_coarse_level(m2)[0] == 5 and m2.level == 5


class FakeEnsemble(object):
    def __init__(self, cost):
        self.cost = cost
        self.offset, self.structure = 0, (0, None)
        self.log = []

    def free_batch(self):
        self.structure = (0, None)

    def coarse_offset(self, d):
        self.offset = d

    def capture(self):
        self.log.append("capture")

    def build_batch(self, groups, policy):
        self.structure = (groups, policy)

    def run(self, n):
        pass


def test_ensemble_keeps_the_fastest_structure(fake_cuda, monkeypatch):
    def cost(e):
        groups, policy = e.structure
        return 10. + (0.5 if e.offset == 0 else 0.) + abs(groups - 8) * 0.1 + (policy == 0) * 0.3

    E = FakeEnsemble(cost)
    monkeypatch.setattr(autotune, "_time", lambda run, steps, warmup: cost(E))
    best, times = autotune.tune_ensemble(E)
    assert best == (1, 8, 1)
    assert (E.offset, E.structure) == (1, (8, 1))
    assert len(times) == 2 * 7          # per offset: stream replay + 6 batched candidates


def test_ensemble_may_keep_stream_replay(fake_cuda, monkeypatch):
    E = FakeEnsemble(None)
    monkeypatch.setattr(autotune, "_time",
                        lambda run, steps, warmup: 1.0 if E.structure[0] == 0 else 2.0)
    best, _ = autotune.tune_ensemble(E, offsets=(0,))
    assert best == (0, 0, None) and E.structure == (0, None)
