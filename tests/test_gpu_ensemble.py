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


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("groups,policy", [(1, 1), (2, 0)])
def test_batched_launches_equal_each_instance_alone(precision, groups, policy):
    """The batched step (one launch per kernel for a group of instances,
    merged from the recorded per-instance steps) reproduces every instance's
    own step, with instances of different sizes, masks and models: bit for
    bit in the exact build (the same body code; the product build may
    contract multiply-adds differently in the batched kernels)."""
    import torch
    from fluid2d_gb300 import engine, workloads as W
    wls = W.ensemble(5, seed=23, nmin=64, nmax=320)
    wls.append(W.shear(128, 64, seed=4, delta=0.1))
    wls.append(W.turbulence(64, 64, seed=6))
    batched = engine.ensemble_from_workloads(wls, precision=precision, batched=True,
                                             groups=groups, policy=policy, variant="exact")
    launches, ops = batched.batch_info()
    assert 0 < launches < ops
    batched.run(4)
    torch.cuda.synchronize()
    for k, wl in enumerate(wls):
        alone = engine.ensemble_from_workloads([wl], precision=precision, nstreams=1,
                                               variant="exact")
        alone.models[0].run(4)
        torch.cuda.synchronize()
        assert torch.equal(alone.models[0].var.state, batched.models[k].var.state), k
        assert torch.equal(alone.models[0]._diag, batched.models[k]._diag), k


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_product_with_coarse_operators(precision):
    """Product build: batched groups dealt round-robin, with every instance's
    coarse part applied as its precomputed operator (the batched form of
    the operator launch) and the coarse switch moved one level down, agree
    with each instance run alone to rounding."""
    import numpy as np
    import torch
    from fluid2d_gb300 import engine, workloads as W
    wls = W.ensemble(4, seed=29, nmin=64, nmax=256)
    wls.append(W.turbulence(128, 128, seed=8))
    E = engine.ensemble_from_workloads(wls, precision=precision)
    assert all(m.coarse_operator() > 0 for m in E.models)
    E.coarse_offset(1)
    E.build_batch(2, 1, balanced=True)
    launches, ops = E.batch_info()
    assert 0 < launches < ops
    E.run(3)
    torch.cuda.synchronize()
    for k, wl in enumerate(wls):
        M = engine.ensemble_from_workloads([wl], precision=precision, nstreams=1).models[0]
        cur, first, nlev = M.coarse_switch()
        M.coarse_switch(min(first + 1, nlev))
        M.run(3)
        torch.cuda.synchronize()
        a, b = M.var.state.cpu().numpy(), E.models[k].var.state.cpu().numpy()
        for v in range(a.shape[0]):
            err = np.abs(a[v] - b[v]).max() / max(1e-300, np.abs(a[v]).max())
            assert err <= 1e-10, (k, v, err)


@pytest.mark.parametrize("batched", [False, True])
def test_failing_instances_are_retired_alone(batched):
    """One instance starts with a NaN in its vorticity, another with a
    velocity beyond the reference's blow-up threshold (maxspeed > 1e3,
    core/fluid2d.py:309-314): the status words retire exactly those two, and
    the others go on bit for bit as they do alone (exact build)."""
    import torch
    from fluid2d_gb300 import engine, workloads as W
    wls = W.ensemble(5, seed=24, nmin=64, nmax=192)
    E = engine.ensemble_from_workloads(wls, batched=batched, groups=2, variant="exact",
                                       nstreams=4)
    bad_nan, bad_fast = E.models[1], E.models[3]
    w = bad_nan.get("vorticity")
    w[10, 10] = float("nan")
    bad_fast.get("psi").mul_(1e7)
    bad_fast.get("u").mul_(1e7)
    bad_fast.get("v").mul_(1e7)
    torch.cuda.synchronize()
    if batched:  # record the batch after the states were changed (no effect on it)
        E.build_batch(2, 1)
    gone = E.run(2, check=True)
    assert sorted(id(m) for m, _ in gone) == sorted([id(bad_nan), id(bad_fast)])
    bits = {id(m): st for m, st in gone}
    assert bits[id(bad_nan)] & 1
    assert bits[id(bad_fast)] & 2
    assert len(E.models) == 3 and not E.run(2, check=True)
    torch.cuda.synchronize()
    keep = [0, 2, 4]
    for k, m in zip(keep, E.models):
        alone = engine.ensemble_from_workloads([wls[k]], nstreams=1, variant="exact")
        alone.models[0].run(4)
        torch.cuda.synchronize()
        assert torch.equal(alone.models[0].var.state, m.var.state), k
        assert m.status() == 0
