"""Parity at the sizes of the named workloads, against the CPU oracle.

* Euler dipole, closed 128x128 (the reference's CPU-runnable case): the
  exact build is bit-identical to the oracle for 20 steps; the product build
  (FMA contraction, coarse multigrid part as its precomputed operator) stays
  within 1e-10 relative L-inf for all 200 steps of the workload.
* Euler turbulence, periodic 1024x1024: the product build within 1e-10
  relative L-inf of the oracle for omega and psi after each of the first 10
  steps (the parity bar), and u, v likewise.
* Boussinesq shear layer, channel 2048x512, Ri = 0.1: the float64 product
  build within 1e-10 of the oracle for 10 steps (omega, psi, b); one step of
  the mixed form (float32 fluxes and cycles in float64 defect correction)
  from the oracle's state within 1e-6 relative L2 of the oracle's step.

The oracle is the parity reference; every state the GPU computes starts from the
oracle's state (the workload generators use numpy transcendentals, which
round differently on other CPU architectures).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_linf(a, b):
    return float(np.abs(a - b).max() / max(1e-300, np.abs(b).max()))


def rel_l2(a, b):
    return float(np.sqrt(((a - b) ** 2).sum()) / max(1e-300, np.sqrt((b ** 2).sum())))


def pair(wl, variant="product", precision="fp64", **kw):
    """(param, oracle model, GPU model on the oracle's initial state, dt)"""
    import torch
    from fluid2d_gb300 import engine
    from oracle import stepper
    p, O = stepper.from_workload(wl, **kw)
    dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
    G = engine.from_workload(wl, dt=dt, variant=variant, precision=precision, **kw)
    G.var.state.copy_(torch.from_numpy(O.state).cuda())
    G.diagnostics()
    return p, O, G, dt


def test_dipole_128_exact_build_is_bit_identical():
    from fluid2d_gb300 import workloads as W
    from oracle import stepper
    p, O, G, dt = pair(W.dipole(128, 128), variant="exact")
    t = 0.
    for k in range(20):
        t = stepper.run(O, p, 1, dt, t=t)
        G.run(1)
        st = G.var.state.cpu().numpy()
        for q, nm in enumerate(G.var.varname_list):
            assert np.array_equal(st[q], O.state[q]), (k + 1, nm)


def test_dipole_128_200_steps():
    from fluid2d_gb300 import workloads as W
    from oracle import stepper
    p, O, G, dt = pair(W.dipole(128, 128))
    t = 0.
    for k in range(1, 201):
        t = stepper.run(O, p, 1, dt, t=t)
        G.run(1)
        if k % 20 == 0:
            st = G.var.state.cpu().numpy()
            for nm in ("vorticity", "psi", "u", "v"):
                q = G.var.varname_list.index(nm)
                e = rel_linf(st[q], O.state[q])
                assert e <= 1e-10, (k, nm, e)


def test_turbulence_1024_first_10_steps():
    from fluid2d_gb300 import workloads as W
    from oracle import stepper
    p, O, G, dt = pair(W.turbulence(1024, 1024))
    assert G.coarse_operator() > 0  # the product path as benchmarked
    t = 0.
    for k in range(1, 11):
        t = stepper.run(O, p, 1, dt, t=t)
        G.run(1)
        st = G.var.state.cpu().numpy()
        for nm in ("vorticity", "psi", "u", "v"):
            q = G.var.varname_list.index(nm)
            e = rel_linf(st[q], O.state[q])
            assert e <= 1e-10, (k, nm, e)


def test_shear_2048x512_fp64_and_mixed_step():
    import torch
    from fluid2d_gb300 import engine
    from fluid2d_gb300 import workloads as W
    from oracle import stepper
    wl = W.shear(2048, 512)
    p, O, G, dt = pair(wl)
    M = engine.from_workload(wl, dt=dt, precision="mixed")
    names = G.var.varname_list
    t = 0.
    for k in range(1, 11):
        # the mixed form's single step from the oracle's state at step 1
        if k == 1:
            M.var.state.copy_(torch.from_numpy(O.state).cuda())
            M.diagnostics()
        t = stepper.run(O, p, 1, dt, t=t)
        G.run(1)
        st = G.var.state.cpu().numpy()
        for nm in ("vorticity", "psi", "u", "v", "buoyancy"):
            q = names.index(nm)
            e = rel_linf(st[q], O.state[q])
            assert e <= 1e-10, (k, nm, e)
        if k == 1:
            M.run(1)
            sm = M.var.state.cpu().numpy()
            for nm in ("vorticity", "psi", "u", "buoyancy"):
                q = names.index(nm)
                e = rel_l2(sm[q], O.state[q])
                assert e <= 1e-6, ("mixed", nm, e)
