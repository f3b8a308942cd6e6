"""Generate the golden fixtures of tests/golden/ from the reference's own Python.

Run where the reference sources are available (read-only):

    python tests/golden/make_golden.py /path/to/Fluid2d/core

For each case it builds the reference's model (core/grid.py, core/euler.py,
core/boussinesq.py, core/quasigeostrophic.py over core/operators.py,
core/gmg/*.py, core/timescheme.py) with its f2py kernels replaced by the C
oracle (oracle/refshim.py), runs the loop body of core/fluid2d.py:237-268
for a few steps, and checks that oracle/stepper.py -- the restatement the
tests use where the reference is absent -- reproduces every state array and
diagnostic bit for bit.  It then writes the initial state and the states
after each step to <case>.npz.
"""
import contextlib
import io
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fluid2d_gb300 import workloads as W  # noqa: E402
from oracle import refshim, stepper  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
# where this build found the reference sources (read-only)
DEFAULT_CORE = "/root/reference/core"


def cases():
    qg = W.dipole(32, 32, seed=11)
    qg["model"] = "quasigeostrophic"
    qg["fields"] = {"pv": qg["fields"]["vorticity"]}
    isl = W.dipole(48, 32, seed=12)
    isl["Lx"], isl["Ly"] = 1.5, 1.
    jj, ii = np.meshgrid(np.arange(38), np.arange(54), indexing="ij")
    isl["msk"][(jj - 20) ** 2 + (ii - 30) ** 2 < 16] = 0
    isl["fields"]["vorticity"] = isl["fields"]["vorticity"] * isl["msk"]
    return {
        "euler_closed_32": (W.dipole(32, 32, seed=1), {}),
        "euler_closed_islands_48x32": (isl, {}),
        "euler_perio_32": (W.turbulence(32, 32, seed=5, k0=3.), {}),
        "boussinesq_xchannel_64x16": (W.shear(64, 16, seed=3, delta=0.1), {}),
        "qg_closed_32": (qg, {"Rd": 0.3, "beta": 2.0}),
    }


def reference_model(core, wl, kw):
    over = dict(modelname=wl["model"], nx=wl["nx"], ny=wl["ny"], Lx=wl["Lx"], Ly=wl["Ly"],
                geometry=wl["geometry"], gravity=wl.get("gravity", 1.), adaptable_dt=False,
                **kw)
    p = refshim.reference_param(core, **over)
    import grid as rgrid
    with contextlib.redirect_stdout(io.StringIO()):
        g = rgrid.Grid(p)
        g.msk[:] = wl["msk"]
        g.finalize_msk()
        if wl["model"] == "euler":
            import euler
            M = euler.Euler(p, g)
        elif wl["model"] == "boussinesq":
            import boussinesq
            M = boussinesq.Boussinesq(p, g)
        else:
            import quasigeostrophic
            M = quasigeostrophic.QG(p, g)
        for name, f in wl["fields"].items():
            M.var.get(name)[:] = f
        if wl["model"] == "quasigeostrophic":
            M.var.get("pv")[:] += M.pvback
            M.set_psi_from_pv()
        else:
            M.set_psi_from_vorticity()
        M.diagnostics(M.var, 0.)
    return M


def main(core, steps=4):
    for name, (wl, kw) in cases().items():
        R = reference_model(core, wl, kw)
        p, O = stepper.from_workload(wl, **kw)
        assert np.array_equal(R.var.state, O.state), name
        dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
        states = [O.state.copy()]
        diags = [[O.diags[k] for k in sorted(O.diags)]]
        t = 0.
        for k in range(steps):
            R.ope.cst[3] = R.diags["maxspeed"]
            with contextlib.redirect_stdout(io.StringIO()):
                R.step(t, dt)
                R.diagnostics(R.var, t + dt)
            t = stepper.run(O, p, 1, dt, t=t)
            assert np.array_equal(R.var.state, O.state), (name, k)
            for key in O.diags:
                assert float(np.asarray(R.diags[key]).ravel()[0]) == O.diags[key], (name, k, key)
            states.append(O.state.copy())
            diags.append([O.diags[key] for key in sorted(O.diags)])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), msk=wl["msk"],
                            states=np.array(states), diags=np.array(diags),
                            diag_names=np.array(sorted(O.diags)), dt=dt,
                            varnames=np.array(O.varname_list),
                            params=np.array([repr(dict(model=wl["model"], nx=wl["nx"],
                                                       ny=wl["ny"], Lx=wl["Lx"], Ly=wl["Ly"],
                                                       geometry=wl["geometry"],
                                                       gravity=wl.get("gravity", 1.), **kw))]))
        print("%-28s ok: reference == oracle stepper, bit for bit, %d steps" % (name, steps))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FLUID2D_CORE", DEFAULT_CORE))
