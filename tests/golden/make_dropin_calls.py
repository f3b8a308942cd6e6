"""Record how the reference's own Python calls its f2py kernels, and check
that oracle/stepper.py makes the same calls.

Run where the reference sources are available (read-only):

    python tests/golden/make_dropin_calls.py /path/to/Fluid2d/core

For every step fixture of tests/golden/ (made by make_golden.py) it builds
the reference's model over the C oracle (oracle/refshim.py) on the
fixture's initial state -- grid, mask, no-slip walls and islands' arrays
from the fixture, no initial inversion -- and runs the fixture's steps,
recording each call into the five f2py modules (fortran_advection,
fortran_fluxes, fortran_operators, fortran_diag, gmg.fortran_multigrid)
with the kind of each argument: dtype, rank and memory order of arrays (a
strided view is passed differently from a contiguous one), 'scalar' for
numbers.  The reference must reproduce the fixture's states bit for bit,
and the oracle stepper (stepper.from_fixture) must issue the identical
sequence of calls.

dropin_calls.json keeps, per fixture, the number of calls, a sha256 of the
whole sequence and the distinct (routine, argument kinds) forms.  The GPU
drop-in test runs the stepper over the GB300 modules of
fluid2d_gb300/f2py_compat on the same fixtures and checks that it makes this
very sequence; the reference's Python itself cannot run where the GPU is
(its sources are not there), so this file carries its call pattern.
"""
import contextlib
import glob
import io
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))

from oracle import oracle as OK, refshim, stepper  # noqa: E402

OUT = os.path.join(HERE, "dropin_calls.json")


def fixtures():
    """{name: path} of the step fixtures"""
    return {os.path.basename(p)[:-4]: p
            for p in sorted(glob.glob(os.path.join(HERE, "*.npz")))
            if not os.path.basename(p).startswith(("loop_", "fluxes_"))}


def oracle_modules():
    """{f2py module name: namespace of oracle functions under the routine names}"""
    import types
    return {mod: types.SimpleNamespace(**{r: getattr(OK, o) for r, o in names.items()})
            for mod, names in refshim.F2PY_NAMES.items()}


def reference_from_fixture(core, z, **kw):
    """The reference's model on the fixture's initial state (as
    stepper.from_fixture builds the stepper's); ``kw`` overrides Param."""
    p0 = stepper.fixture_param(z)
    over = {k: v for k, v in vars(p0).items() if k not in ("npx", "npy")}
    over["isisland"] = "rhsp" in z
    over.update(kw)
    p = refshim.reference_param(core, **over)
    import grid as rgrid
    with contextlib.redirect_stdout(io.StringIO()):
        g = rgrid.Grid(p)
        g.msk[:] = z["msk"]
        if "msknoslip" in z:
            g.msknoslip[:] = z["msknoslip"]
        g.finalize_msk()
        if p.modelname == "euler":
            import euler
            M = euler.Euler(p, g)
        elif p.modelname == "boussinesq":
            import boussinesq
            M = boussinesq.Boussinesq(p, g)
        else:
            import quasigeostrophic
            M = quasigeostrophic.QG(p, g)
        if "rhsp" in z:
            M.ope.rhsp = np.array(z["rhsp"])
            M.ope.psi = np.array(z["psi_island"])
        M.var.state[...] = z["states"][0]
        M.diagnostics(M.var, 0.)
    return M


# the time schemes of core/timescheme.py:78-201 other than RK3_SSP, replayed
# from one fixture's initial state
SCHEMES = ["EF", "LF", "Heun", "AB2", "AB3", "LFAM3", "RK3", "RK4_LS"]
SCHEME_FIXTURE = "euler_closed_32"
SCHEME_STEPS = 3


def trace_fixture(core, path, timestepping=None, nsteps=None):
    """(reference trace, stepper trace, final state) replaying one fixture,
    with its own time scheme (the fixture's states are checked at every
    step) or another one (the final states are compared)."""
    z = np.load(path, allow_pickle=False)
    states, dt = z["states"], float(z["dt"])
    nsteps = nsteps or len(states) - 1
    over = {"timestepping": timestepping} if timestepping else {}
    refshim.install(core)
    refshim.TRACE.calls = []
    refshim.TRACE.on = True
    try:
        R = reference_from_fixture(core, z, **over)
        t = 0.
        for k in range(1, nsteps + 1):
            R.ope.cst[3] = R.diags["maxspeed"]
            with contextlib.redirect_stdout(io.StringIO()):
                R.step(t, dt)
                R.diagnostics(R.var, t + dt)
            t += dt
            if not timestepping:
                assert np.array_equal(R.var.state, states[k]), (path, k)
    finally:
        refshim.TRACE.on = False
    ref = refshim.CallTrace()
    ref.calls = list(refshim.TRACE.calls)

    mine = refshim.CallTrace()
    old = stepper.use_kernels(refshim.kernel_set(oracle_modules(), mine))
    try:
        p, O = stepper.from_fixture(z, **over)
        stepper.run(O, p, nsteps, dt)
    finally:
        stepper.use_kernels(old)
    assert np.array_equal(O.state, R.var.state), path
    return ref, mine


def first_difference(a, b):
    for k, (x, y) in enumerate(zip(a, b)):
        if x != y:
            return k, x, y
    return min(len(a), len(b)), None, None


def record(core, path, timestepping=None, nsteps=None):
    """The reference's calls replaying one fixture, checked equal to the
    stepper's."""
    ref, mine = trace_fixture(core, path, timestepping, nsteps)
    if ref.calls != mine.calls:
        k, x, y = first_difference(ref.calls, mine.calls)
        raise AssertionError("%s: call %d differs (of %d / %d): reference %r, stepper %r"
                             % (path, k, len(ref.calls), len(mine.calls), x, y))
    return {"calls": len(ref.calls), "sha256": ref.digest(), "forms": ref.forms()}


def main(core):
    out = {}
    fx = fixtures()
    for name, path in fx.items():
        out[name] = record(core, path)
        print("%-40s %5d calls, %2d forms: reference == stepper"
              % (name, out[name]["calls"], len(out[name]["forms"])))
    for scheme in SCHEMES:
        key = "%s:%s" % (SCHEME_FIXTURE, scheme)
        out[key] = record(core, fx[SCHEME_FIXTURE], scheme, SCHEME_STEPS)
        out[key]["steps"] = SCHEME_STEPS
        print("%-40s %5d calls, %2d forms: reference == stepper"
              % (key, out[key]["calls"], len(out[key]["forms"])))
    with open(OUT, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
        f.write("\n")


if __name__ == "__main__":
    core = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FLUID2D_CORE")
    if not core:
        sys.exit("usage: make_dropin_calls.py <reference core/ directory> (or FLUID2D_CORE)")
    main(core)
