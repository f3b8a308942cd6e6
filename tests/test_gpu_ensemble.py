"""Batched ensemble: instances stepped together give exactly what they give
alone (instances share no data; every kernel is deterministic)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_alone_equals_in_the_mix(precision):
    import torch
    from fluid2d_gb300 import engine, workloads as W
    wls = W.ensemble(6, seed=21, nmin=64, nmax=256)
    ens = engine.ensemble_from_workloads(wls, precision=precision, nstreams=4)
    ens.run(5)
    torch.cuda.synchronize()
    mixed_states = [m.var.state.cpu().numpy() for m in ens.models]
    for k in (0, 3, 5):
        alone = engine.ensemble_from_workloads([wls[k]], precision=precision, nstreams=1)
        alone.run(5)
        torch.cuda.synchronize()
        assert np.array_equal(alone.models[0].var.state.cpu().numpy(), mixed_states[k]), k


def test_lockstep_equals_free_running():
    import torch
    from fluid2d_gb300 import engine, workloads as W
    wls = W.ensemble(4, seed=22, nmin=64, nmax=192)
    a = engine.ensemble_from_workloads(wls, nstreams=4)
    b = engine.ensemble_from_workloads(wls, nstreams=2)
    a.run(3)
    b.run(3, lockstep=True)
    torch.cuda.synchronize()
    for ma, mb in zip(a.models, b.models):
        assert torch.equal(ma.var.state, mb.var.state)
