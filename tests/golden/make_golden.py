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


def channel_with_islands(model="euler", nx=64, ny=32, seed=9):
    """A channel with a disc obstacle held at psi = 0 and the walls held at
    +-0.1: a through-flow, as experiments/VonKarman/karman_street.py sets it
    up (islands, no-slip on the disc, free slip on the walls)."""
    Lx, Ly, nh = 2., 1., 3
    msk = W.base_mask(nx, ny, "xchannel")
    xr, yr = W.cell_coords(nx, ny, Lx, Ly)
    disc = np.where(np.sqrt((xr - 0.5) ** 2 + (yr - 0.5) ** 2) <= 0.12)
    msk[disc] = 0
    noslip = W.base_mask(nx, ny, "xchannel")
    noslip[disc] = 0
    noslip[:nh, :] = 1
    noslip[-nh:, :] = 1
    m = np.zeros_like(msk)
    m[:nh, :] = 1
    bottom = np.where(m == 1)
    m = np.zeros_like(msk)
    m[-nh:-1, :] = 1
    top = np.where(m == 1)
    w = 1e-2 * np.random.default_rng(seed).standard_normal(msk.shape)
    w[:, :nh] = w[:, -2 * nh:-nh]  # periodic in x
    w[:, -nh:] = w[:, nh:2 * nh]
    w = w * msk
    name = "pv" if model == "quasigeostrophic" else "vorticity"
    return {"model": model, "geometry": "xchannel", "nx": nx, "ny": ny, "Lx": Lx, "Ly": Ly,
            "msk": msk, "msknoslip": noslip, "fields": {name: w},
            "islands": [(disc, 0.), (bottom, 0.1), (top, -0.1)]}


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
        # diffusion at the forcing stage (core/operators.py:292-300)
        "euler_closed_32_diffusion": (W.dipole(32, 32, seed=1),
                                      {"diffusion": True, "Kdiff": 2e-3}),
        "boussinesq_xchannel_64x16_diffusion": (W.shear(64, 16, seed=3, delta=0.1),
                                                {"diffusion": True, "Kdiff": 1e-3}),
        "qg_closed_32_diffusion": (qg, {"Rd": 0.3, "beta": 2.0, "diffusion": True,
                                        "Kdiff": 2e-3}),
        # no-slip walls (core/operators.py:245-290), with islands in the mask
        # that keep free slip (core/grid.py:101)
        "euler_closed_islands_48x32_noslip": (isl, {"noslip": True}),
        "boussinesq_xchannel_64x16_noslip": (W.shear(64, 16, seed=3, delta=0.1),
                                             {"noslip": True}),
        "qg_closed_32_noslip": (qg, {"Rd": 0.3, "beta": 2.0, "noslip": True}),
        # line relaxation on every level (hydroepsilon*dy/dx <= 0.2,
        # core/gmg/level.py:153-163): flat cells, and a small hydroepsilon
        "euler_closed_16x96_tridiag": (W.dipole(16, 96, seed=4), {}),
        "boussinesq_xchannel_64x16_hydro": (W.shear(64, 16, seed=3, delta=0.1),
                                            {"hydroepsilon": 0.1}),
        # centred fluxes (core/fortran_advection.f90:169-284) and the other
        # upwind orders and flux splitting
        "euler_closed_32_order4": (W.dipole(32, 32, seed=6), {"order": 4}),
        "euler_perio_32_order3_minmax": (W.turbulence(32, 32, seed=7, k0=3.),
                                         {"order": 3, "flux_splitting_method": "minmax"}),
        "boussinesq_xchannel_64x16_order2": (W.shear(64, 16, seed=8, delta=0.1),
                                             {"order": 2}),
        # islands with a prescribed streamfunction (core/island.py)
        "euler_xchannel_64x32_islands_noslip": (channel_with_islands(), {"noslip": True}),
        "qg_xchannel_64x32_islands": (channel_with_islands("quasigeostrophic"),
                                      {"Rd": 0.5, "beta": 1.0}),
    }


def reference_model(core, wl, kw, with_param=False):
    over = dict(modelname=wl["model"], nx=wl["nx"], ny=wl["ny"], Lx=wl["Lx"], Ly=wl["Ly"],
                geometry=wl["geometry"], gravity=wl.get("gravity", 1.), adaptable_dt=False,
                isisland=bool(wl.get("islands")))
    over.update(kw)
    p = refshim.reference_param(core, **over)
    import grid as rgrid
    with contextlib.redirect_stdout(io.StringIO()):
        g = rgrid.Grid(p)
        g.msk[:] = wl["msk"]
        if "msknoslip" in wl:
            g.msknoslip[:] = wl["msknoslip"]
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
        if wl.get("islands"):  # core/fluid2d.py:110-113
            for idx, psi0 in wl["islands"]:
                g.island.add(idx, psi0)
            g.island.finalize(M.ope.mskp)
            M.ope.rhsp = g.island.rhsp
            M.ope.psi = g.island.psi
        for name, f in wl["fields"].items():
            M.var.get(name)[:] = f
        if wl["model"] == "quasigeostrophic":
            M.var.get("pv")[:] += M.pvback
            M.set_psi_from_pv()
        else:
            M.set_psi_from_vorticity()
        M.diagnostics(M.var, 0.)
    if with_param:
        return M, p, g
    return M


# ---------------------------------------------------------------- time loop
LOOP_CASES = {
    # adaptive dt with the exact-history-time countdown; two saved planes
    "loop_euler_closed_32": (lambda: W.dipole(32, 32, seed=1),
                             dict(adaptable_dt=True, cfl=0.8, dt=0.1, dtmax=5.),
                             dict(tend=0.2, freq_his=0.05, freq_diag=0.02,
                                  var_to_save=["vorticity", "psi"], exacthistime=True)),
    # fixed dt (no countdown), Boussinesq, history times crossed between steps
    "loop_boussinesq_xchannel_64x16": (lambda: W.shear(64, 16, seed=3, delta=0.1),
                                       dict(adaptable_dt=False, dt=0.004),
                                       dict(tend=0.1, freq_his=0.03, freq_diag=0.01,
                                            var_to_save=["vorticity", "buoyancy"],
                                            exacthistime=True)),
    # flux diagnostic at every history record (adaptive dt, countdown)
    "loop_boussinesq_xchannel_64x16_fluxes": (lambda: W.shear(64, 16, seed=3, delta=0.1),
                                              dict(adaptable_dt=True, cfl=0.8, dt=0.1,
                                                   dtmax=5.),
                                              dict(tend=0.06, freq_his=0.02, freq_diag=0.01,
                                                   var_to_save=["vorticity"],
                                                   exacthistime=True, diag_fluxes=True)),
    # time rescaled by the enstrophy, adaptive dt without the countdown
    "loop_euler_perio_32_rescaled": (lambda: W.turbulence(32, 32, seed=5, k0=3.),
                                     dict(adaptable_dt=True, cfl=0.6, dt=0.1, dtmax=5.),
                                     dict(tend=0.4, freq_his=0.1, freq_diag=0.05,
                                          var_to_save=["vorticity"], exacthistime=False,
                                          rescaledtime="enstrophy")),
}


def reference_loop(core, wl, kw, lk, tmpdir):
    """Fluid2d.loop (core/fluid2d.py:190-330) of the reference, run on an
    object holding only the attributes the loop reads (the rest of
    Fluid2d.__init__ copies scripts and redirects stdout), with the
    reference's own Output writing into the in-memory netCDF recorder."""
    import types
    R, p, g = reference_model(core, wl, kw, with_param=True)
    init_state = R.var.state.copy()
    # the domain area is a size-1 array there (core/grid.py domain_integration
    # over mpitools), which makes every diagnostic a size-1 array; numpy 2
    # no longer converts those to the scalars that Output.write_diag stores
    # (core/output.py:132).  A scalar area gives the same quotients.
    R.area = float(np.asarray(R.area).ravel()[0])
    refshim.install_recording_netcdf()
    import fluid2d as rfluid2d
    import output as routput
    routput.Dataset = refshim.RecordingDataset
    p.expname = "loop"
    p.expdir = tmpdir
    p.tend = lk["tend"]
    p.freq_his = lk["freq_his"]
    p.freq_diag = lk["freq_diag"]
    p.var_to_save = list(lk["var_to_save"])
    p.list_diag = "all"
    p.nprint = 10 ** 9
    flx = None
    if lk.get("diag_fluxes"):
        import fluxes as rfluxes
        p.diag_fluxes = True
        flx = rfluxes.Fluxes(p, g, R.ope)
    with contextlib.redirect_stdout(io.StringIO()):
        out = routput.Output(p, g, R.diags,
                             flxlist=flx.fullflx_list if flx is not None else None)
    F = types.SimpleNamespace(
        myrank=0, decay=False, modelname=wl["model"], model=R, diag_fluxes=flx is not None,
        flx=flx, output=out,
        plot_interactive=False, nh=3, t=0., kt=0, tend=lk["tend"],
        exacthistime=lk["exacthistime"], adaptable_dt=kw["adaptable_dt"], dt=kw["dt"],
        dt0=kw["dt"], cfl=p.cfl, dtmax=p.dtmax, dx=g.dx, dy=g.dy, rescaledtime=lk.get("rescaledtime", "none"),
        enstrophyname="enstrophy", enforce_momentum=False, nprint=10 ** 9, freq_plot=10 ** 9,
        npx=1, npy=1, nx=wl["nx"], ny=wl["ny"], nbproc=1)
    F.set_dt = lambda kt: rfluid2d.Fluid2d.set_dt(F, kt)
    F.print_config = lambda *a, **k: None
    with contextlib.redirect_stdout(io.StringIO()):
        rfluid2d.Fluid2d.loop(F)
    files = refshim.RecordingDataset.FILES
    his = files[out.hisfile]["variables"]
    dia = files[out.diagfile]["variables"]
    his = {k: v.a for k, v in his.items()}
    if flx is not None:
        his.update({"flx:" + k: v.a for k, v in files[out.flxfile]["variables"].items()})
    return R, his, {k: v.a for k, v in dia.items()}, init_state


def main_loop(core):
    import tempfile
    refshim.install(core)
    refshim.install_recording_netcdf()
    for name, (mk, kw, lk) in LOOP_CASES.items():
        wl = mk()
        with tempfile.TemporaryDirectory() as tmp:
            R, his, dia, R0_state = reference_loop(core, wl, kw, lk, tmp)
        p, O = stepper.from_workload(wl, **kw)
        # the initial state is stored: numpy's transcendental ufuncs (exp,
        # tanh, ...) round differently on other CPU architectures, so the
        # workload generators are not bit-reproducible across machines
        init_state = O.state.copy()
        assert np.array_equal(R0_state, init_state), name
        fl = stepper.Fluxes(O) if lk.get("diag_fluxes") else None
        out = stepper.History(lk["var_to_save"], lk["freq_his"], lk["freq_diag"], fluxes=fl)
        t, kt, dts, reason = stepper.loop(O, p, lk["tend"], kw["dt"], out,
                                          exacthistime=lk["exacthistime"],
                                          rescaledtime=lk.get("rescaledtime", "none"))
        assert np.array_equal(R.var.state, O.state), name
        assert np.array_equal(his["t"], np.array([h[0] for h in out.his], np.float32)), name
        assert np.array_equal(his["kt"], np.array([h[1] for h in out.his], np.int32)), name
        for v in lk["var_to_save"]:
            assert np.array_equal(his[v], np.array([h[2][v] for h in out.his])), (name, v)
        assert np.array_equal(dia["t"], np.array([d[0] for d in out.diag], np.float32)), name
        assert np.array_equal(dia["kt"], np.array([d[1] for d in out.diag], np.int32)), name
        names = [k for k in out.diag[0][2]]
        for k in names:
            assert np.array_equal(dia[k], np.array([d[2][k] for d in out.diag], np.float32)), \
                (name, k)
        fx = dict(msk=wl["msk"], his_t=his["t"], his_kt=his["kt"],
                  his_t64=np.array([h[0] for h in out.his]),
                  diag_t=dia["t"], diag_kt=dia["kt"], diag_names=np.array(names),
                  diag=np.array([dia[k] for k in names]).T,
                  diag64=np.array([[d[2][k] for k in names] for d in out.diag]),
                  dts=np.array(dts), init_state=init_state, final_state=O.state,
                  var_to_save=np.array(lk["var_to_save"]),
                  params=np.array([repr(dict(model=wl["model"], nx=wl["nx"], ny=wl["ny"],
                                             Lx=wl["Lx"], Ly=wl["Ly"],
                                             geometry=wl["geometry"],
                                             gravity=wl.get("gravity", 1.), **kw))]),
                  loop=np.array([repr(lk)]))
        for v in lk["var_to_save"]:
            fx["his_" + v] = his[v]
        if fl is not None:
            assert np.array_equal(his["flx:t"], fx["his_t"]), name
            assert np.array_equal(his["flx:kt"], fx["his_kt"]), name
            for v in fl.fullflx_list:
                assert np.array_equal(his["flx:" + v],
                                      np.array([f[2][v] for f in out.flx])), (name, v)
            fx["flx_names"] = np.array(fl.fullflx_list)
            fx["flx"] = np.array([[f[2][v] for v in fl.fullflx_list] for f in out.flx])
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **fx)
        print("%-28s ok: reference loop == oracle loop, %d steps, %d records, %d rows"
              % (name, kt, len(out.his), len(out.diag)))


def main(core, steps=4):
    from fluid2d_gb300.island import Island
    for name, (wl, kw) in cases().items():
        R = reference_model(core, wl, kw)
        extra = {}
        if wl.get("islands"):
            # the product's host restatement of core/island.py gives the same arrays
            I = Island(wl["nx"] + 6, wl["ny"] + 6, wl["Lx"] / wl["nx"], wl["Ly"] / wl["ny"])
            for idx, psi0 in wl["islands"]:
                I.add(idx, psi0)
            rhsp, psi = I.finalize()
            assert np.array_equal(rhsp, R.ope.rhsp) and np.array_equal(psi, R.ope.psi), name
            wl = dict(wl, island_arrays=(rhsp, psi))
            extra = dict(rhsp=rhsp, psi_island=psi)
        if "msknoslip" in wl:
            extra["msknoslip"] = wl["msknoslip"]
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
        np.savez_compressed(os.path.join(HERE, name + ".npz"), msk=wl["msk"], **extra,
                            states=np.array(states), diags=np.array(diags),
                            diag_names=np.array(sorted(O.diags)), dt=dt,
                            varnames=np.array(O.varname_list),
                            params=np.array([repr(dict(model=wl["model"], nx=wl["nx"],
                                                       ny=wl["ny"], Lx=wl["Lx"], Ly=wl["Ly"],
                                                       geometry=wl["geometry"],
                                                       gravity=wl.get("gravity", 1.), **kw))]))
        print("%-28s ok: reference == oracle stepper, bit for bit, %d steps" % (name, steps))


# ------------------------------------------------------ flux diagnostics
FLUX_CASES = {
    "fluxes_euler_closed_32": lambda: W.dipole(32, 32, seed=1),
    "fluxes_boussinesq_xchannel_64x16": lambda: W.shear(64, 16, seed=3, delta=0.1),
}


def main_fluxes(core, steps=2):
    """Fluxes.diag_fluxes (core/fluxes.py:100-170) of the reference, on the
    reference model's state after each of `steps` steps, against the oracle's
    restatement (stepper.Fluxes), bit for bit."""
    refshim.install(core)
    for name, mk in FLUX_CASES.items():
        wl = mk()
        R, p, g = reference_model(core, wl, {}, with_param=True)
        import fluxes as rfluxes
        F = rfluxes.Fluxes(p, g, R.ope)
        pO, O = stepper.from_workload(wl)
        init_state = O.state.copy()
        assert np.array_equal(R.var.state, init_state), name
        OF = stepper.Fluxes(O)
        assert OF.fullflx_list == list(F.fullflx_list), name
        dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
        t = 0.
        flx = []
        for k in range(steps):
            R.ope.cst[3] = R.diags["maxspeed"]
            with contextlib.redirect_stdout(io.StringIO()):
                R.step(t, dt)
                R.diagnostics(R.var, t + dt)
            t = stepper.run(O, pO, 1, dt, t=t)
            assert np.array_equal(R.var.state, O.state), (name, k)
            F.diag_fluxes(R.var.state, t, dt)
            OF.diag_fluxes(O.state, t, dt)
            assert np.array_equal(F.flx, OF.flx), (name, k)
            assert np.array_equal(R.var.state, O.state), (name, k)
            flx.append(OF.flx.copy())
        np.savez_compressed(os.path.join(HERE, name + ".npz"), msk=wl["msk"],
                            init_state=init_state, dt=dt, flx=np.array(flx),
                            final_state=O.state, names=np.array(OF.fullflx_list),
                            model=np.array([wl["model"]]))
        print("%-34s ok: reference Fluxes == oracle Fluxes, bit for bit, %d calls"
              % (name, steps))


if __name__ == "__main__":
    # the reference's core/ directory (read-only), from the command line or
    # the FLUID2D_CORE environment variable
    core = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FLUID2D_CORE")
    if not core:
        sys.exit("usage: make_golden.py <reference core/ directory> (or FLUID2D_CORE)")
    main(core)
    main_loop(core)
    main_fluxes(core)
