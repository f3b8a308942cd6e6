"""The reference's Python sequencing run unchanged over the GB300 drop-in
modules (fluid2d_gb300/f2py_compat: fortran_advection, fortran_fluxes,
fortran_operators, fortran_diag, gmg.fortran_multigrid).

The reference's own core/*.py cannot be imported here (its sources do not
travel with the tests), so its sequencing is the oracle's restatement,
oracle/stepper.py, which tests/golden/make_dropin_calls.py pinned to it
where the reference was present: replaying each step fixture, the
reference's euler.py / boussinesq.py / quasigeostrophic.py over
operators.py, gmg/*.py and timescheme.py make exactly the stepper's kernel
calls (same routines, same order, same array dtypes, ranks and memory
orders), recorded in tests/golden/dropin_calls.json with a sha256 of each
whole sequence.

Here the stepper calls the GPU modules instead of the oracle:

* every step fixture (Euler, Boussinesq, QG; closed, periodic and channel
  domains; islands, no-slip walls, diffusion, line relaxation, centred and
  third-order advection) reproduces the fixture's states -- bit for bit in
  the exact build, within 1e-10 of the largest value in the product build --
  and the call sequence hashes to the reference's;
* the other time schemes of core/timescheme.py:78-201 (EF, LF, Heun, AB2,
  AB3, LFAM3, RK3, RK4_LS) give the oracle's states over three steps, with
  the reference's call sequence.

Arrays are numpy arrays, as the reference passes them: every call takes
the host-buffer path (copied to the GPU and back).
"""
import glob
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
FIXTURES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz"))
                  if not os.path.basename(p).startswith(("loop_", "fluxes_")))
SCHEMES = ["EF", "LF", "Heun", "AB2", "AB3", "LFAM3", "RK3", "RK4_LS"]


def calls():
    with open(os.path.join(GOLDEN, "dropin_calls.json")) as f:
        return json.load(f)


def gpu_modules():
    """the drop-in modules, by the names the reference imports"""
    from fluid2d_gb300.f2py_compat import (fortran_advection, fortran_diag, fortran_fluxes,
                                           fortran_operators)
    from fluid2d_gb300.f2py_compat.gmg import fortran_multigrid
    return {"fortran_advection": fortran_advection, "fortran_fluxes": fortran_fluxes,
            "fortran_operators": fortran_operators, "fortran_diag": fortran_diag,
            "gmg.fortran_multigrid": fortran_multigrid}


@pytest.fixture
def over_gpu():
    """Run oracle/stepper.py over the GPU modules, traced; restore after."""
    from fluid2d_gb300 import kernels
    from oracle import refshim, stepper
    state = {}

    def use(variant):
        state["variant"] = kernels.use_variant(variant)
        trace = refshim.CallTrace()
        state["kernels"] = stepper.use_kernels(refshim.kernel_set(gpu_modules(), trace))
        return trace

    yield use
    if "kernels" in state:
        stepper.use_kernels(state["kernels"])
    if "variant" in state:
        kernels.use_variant(state["variant"])


@pytest.mark.parametrize("variant", ["exact", "product"])
@pytest.mark.parametrize("name", FIXTURES)
def test_reference_sequencing_over_gpu_modules(name, variant, over_gpu):
    from oracle import stepper
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    states, dt = z["states"], float(z["dt"])
    trace = over_gpu(variant)
    p, M = stepper.from_fixture(z)
    t = 0.
    for k in range(1, len(states)):
        t = stepper.run(M, p, 1, dt, t=t)
        for q, nm in enumerate(M.varname_list):
            if variant == "exact":
                assert np.array_equal(M.state[q], states[k][q]), (k, nm)
            else:
                scale = max(np.abs(states[k][q]).max(), 1e-300)
                assert np.abs(M.state[q] - states[k][q]).max() <= 1e-10 * scale, (k, nm)
    ref = calls()[name]
    assert len(trace.calls) == ref["calls"]
    assert trace.forms() == ref["forms"]
    assert trace.digest() == ref["sha256"]


@pytest.mark.parametrize("scheme", SCHEMES)
def test_time_schemes_over_gpu_modules(scheme, over_gpu):
    """core/timescheme.py keeps working over the GPU modules: the oracle's
    states (bit for bit, exact build) and the reference's calls."""
    from oracle import stepper
    key = "euler_closed_32:%s" % scheme
    ref = calls()[key]
    z = np.load(os.path.join(GOLDEN, "euler_closed_32.npz"), allow_pickle=False)
    dt = float(z["dt"])
    p, O = stepper.from_fixture(z, timestepping=scheme)
    stepper.run(O, p, ref["steps"], dt)
    trace = over_gpu("exact")
    p, M = stepper.from_fixture(z, timestepping=scheme)
    stepper.run(M, p, ref["steps"], dt)
    assert np.array_equal(M.state, O.state)
    assert trace.digest() == ref["sha256"]
    assert not np.array_equal(M.state, z["states"][0])
