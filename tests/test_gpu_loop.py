"""The device-resident time loop against the oracle's Fluid2d.loop.

The loop fixtures of tests/golden/ hold what the reference's own
Fluid2d.loop and Output wrote (history planes in float32, record times and
iterations, diagnostic rows) for three runs: adaptive dt with the
exact-history-time countdown (Euler, closed), fixed dt (Boussinesq,
xchannel), enstrophy-rescaled time (Euler, periodic).  With the exact build
the closed-domain runs are bit-identical to the fixtures (every time step is
cfl*dx/maxspeed of a bit-identical state, and the countdown is the same
arithmetic); the periodic run and the product build are compared with
tolerances.  Diagnostic rows hold sums, whose rounding differs between the
device's tree reduction and the oracle's sequential one.
"""
import ast
import importlib.util
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["loop_euler_closed_32", "loop_boussinesq_xchannel_64x16",
         "loop_boussinesq_xchannel_64x16_fluxes", "loop_euler_perio_32_rescaled"]


def _mg():
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def _fixture(name):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"), allow_pickle=False)
    mk, kw, lk = _mg().LOOP_CASES[name]
    assert lk == ast.literal_eval(str(z["loop"][0]))
    return z, mk(), kw, lk


def _setup_kw(lk, **over):
    d = dict(freq_his=lk["freq_his"], freq_diag=lk["freq_diag"],
             var_to_save=lk["var_to_save"], exacthistime=lk["exacthistime"],
             rescaledtime=lk.get("rescaledtime", "none"),
             diag_fluxes=lk.get("diag_fluxes", False))
    d.update(over)
    return d


def _model(wl, kw, variant, init=None):
    """A device model started from the fixture's initial state (the workload
    generators use numpy's transcendental ufuncs, whose last-bit rounding
    differs between CPU architectures) or from the oracle's."""
    import torch
    from fluid2d_gb300 import engine
    from oracle import stepper
    if init is None:
        p, O = stepper.from_workload(wl, **kw)
        init = O.state
    G = engine.from_workload(wl, variant=variant, **kw)
    G.var.state.copy_(torch.from_numpy(np.ascontiguousarray(init)).cuda())
    return G


def _oracle(wl, kw, init):
    from oracle import stepper
    p, O = stepper.from_workload(wl, **kw)
    O.state[:] = init
    O.diagnostics()
    return p, O


def _assert_state_equal(G, ref):
    st = G.var.state.cpu().numpy()
    bad = []
    for k, nm in enumerate(G.var.varname_list):
        if not np.array_equal(st[k], ref[k]):
            jj, ii = np.nonzero(st[k] != ref[k])
            bad.append((nm, len(jj), sorted(set(jj.tolist()))[:8], sorted(set(ii.tolist()))[:8],
                        float(np.abs(st[k] - ref[k]).max())))
    assert not bad, bad


def _relmax(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() /
                 max(1e-300, np.abs(np.asarray(b)).max()))


@pytest.mark.parametrize("variant", ["exact", "product"])
@pytest.mark.parametrize("name", NAMES)
def test_device_loop_matches_reference_loop(name, variant):
    z, wl, kw, lk = _fixture(name)
    G = _model(wl, kw, variant, z["init_state"])
    st = G.loop(lk["tend"], **_setup_kw(lk))
    assert st["status"] == "tend"
    his, diag = st["his"], st["diag"]
    assert [h[1] for h in his] == list(z["his_kt"])
    t = np.array([h[0] for h in his])
    bitexact = variant == "exact" and wl["geometry"] != "perio" and \
        lk.get("rescaledtime", "none") == "none"
    if bitexact:
        assert np.array_equal(t, z["his_t64"])
        assert np.array_equal(np.array([h[1] for h in his], np.int32), z["his_kt"])
        for v in lk["var_to_save"]:
            assert np.array_equal(np.array([h[2][v] for h in his]), z["his_" + v]), v
        _assert_state_equal(G, z["final_state"])
    else:
        assert _relmax(t, z["his_t64"]) < 1e-12
        for v in lk["var_to_save"]:
            assert _relmax(np.array([h[2][v] for h in his]), z["his_" + v]) < 1e-6, v
        assert _relmax(G.var.state.cpu().numpy()[0], z["final_state"][0]) < 1e-9
    if lk.get("diag_fluxes"):
        fl = [str(n) for n in z["flx_names"]]
        got = np.array([[h[2]["flx:" + v] for v in fl] for h in his])
        if bitexact:
            assert np.array_equal(got, z["flx"])
        else:
            assert _relmax(got, z["flx"]) < 1e-6
    names = [str(n) for n in z["diag_names"]]
    rows = np.array([[d[2][k] for k in names] for d in diag])
    assert rows.shape == z["diag64"].shape
    assert np.array_equal(np.array([d[1] for d in diag], np.int32), z["diag_kt"])
    for q, k in enumerate(names):
        ref = z["diag64"][:, q]
        scale = max(np.abs(ref).max(), 1e-300)
        # sums: relative 1e-10 of the largest value, or 1e-13 absolute for
        # the integrals that vanish up to rounding (mean vorticity of a
        # periodic flow); dkedt, dvdt are differences of sums over dt
        tol = 1e-6 if k in ("dkedt", "dvdt") else 1e-10
        assert np.abs(rows[:, q] - ref).max() <= tol * scale + 1e-13, k


def test_ring_pause_and_resume_change_nothing():
    z, wl, kw, lk = _fixture("loop_euler_closed_32")
    A = _model(wl, kw, "exact", z["init_state"])
    a = A.loop(lk["tend"], **_setup_kw(lk))
    B = _model(wl, kw, "exact", z["init_state"])
    b = B.loop(lk["tend"], **_setup_kw(lk, his_cap=2, diag_cap=3))
    assert [h[:2] for h in a["his"]] == [h[:2] for h in b["his"]]
    for x, y in zip(a["his"], b["his"]):
        for v in lk["var_to_save"]:
            assert np.array_equal(x[2][v], y[2][v])
    assert [d[:2] for d in a["diag"]] == [d[:2] for d in b["diag"]]
    assert np.array_equal(A.var.state.cpu().numpy(), B.var.state.cpu().numpy())


def test_max_steps_bounds_a_launch_and_the_run_continues():
    import torch
    z, wl, kw, lk = _fixture("loop_euler_closed_32")
    G = _model(wl, kw, "exact", z["init_state"])
    G.loop_setup(lk["tend"], **_setup_kw(lk, his_cap=16, diag_cap=64))
    G.loop_start()
    G.loop_run(5)
    s = G.loop_state()
    assert s["kt"] == 5 and s["status"] == "running"
    G.loop_run(1000)
    torch.cuda.synchronize()
    s = G.loop_state()
    assert s["status"] == "tend" and s["kt"] == int(z["his_kt"][-1])
    his, diag = G.loop_drain()
    assert np.array_equal(np.array([h[0] for h in his]), z["his_t64"])
    _assert_state_equal(G, z["final_state"])


def test_blowup_stops_after_one_step():
    from oracle import stepper
    z, wl, kw, lk = _fixture("loop_euler_closed_32")
    wl = dict(wl)
    wl["fields"] = {"vorticity": wl["fields"]["vorticity"] * 1e6}
    G = _model(wl, kw, "exact")
    st = G.loop(lk["tend"], **_setup_kw(lk))
    p, O = stepper.from_workload(wl, **kw)
    out = stepper.History(lk["var_to_save"], lk["freq_his"], lk["freq_diag"])
    t, kt, dts, reason = stepper.loop(O, p, lk["tend"], kw["dt"], out)
    assert reason == "blowup" and kt == 1
    assert st["status"] == "blowup" and st["kt"] == 1
    assert st["t"] == t


def test_output_files_hold_the_records(tmp_path):
    from scipy.io import netcdf_file
    from fluid2d_gb300.output import Output
    z, wl, kw, lk = _fixture("loop_boussinesq_xchannel_64x16")
    G = _model(wl, kw, "exact", z["init_state"])
    out = Output.for_model(G, str(tmp_path), "shear", var_to_save=lk["var_to_save"],
                           param=dict(kw, tend=lk["tend"], modelname="boussinesq"))
    st = G.loop(lk["tend"], output=out, **_setup_kw(lk, his_cap=2))
    assert st["his"] == [] and st["status"] == "tend"
    with netcdf_file(out.hisfile, "r", mmap=False) as nc:
        assert np.array_equal(np.array(nc.variables["kt"][:]), z["his_kt"])
        assert np.array_equal(np.array(nc.variables["t"][:]).astype(np.float32), z["his_t"])
        for v in lk["var_to_save"]:
            assert np.array_equal(np.array(nc.variables[v][:]).astype(np.float32),
                                  z["his_" + v])
    with netcdf_file(out.diagfile, "r", mmap=False) as nc:
        assert np.array_equal(np.array(nc.variables["kt"][:]), z["diag_kt"])


def test_flux_file_holds_the_flux_records(tmp_path):
    from scipy.io import netcdf_file
    from fluid2d_gb300.output import Output
    z, wl, kw, lk = _fixture("loop_boussinesq_xchannel_64x16_fluxes")
    G = _model(wl, kw, "exact", z["init_state"])
    out = Output.for_model(G, str(tmp_path), "shear", var_to_save=lk["var_to_save"],
                           fluxes=True)
    st = G.loop(lk["tend"], output=out, **_setup_kw(lk, his_cap=2))
    assert st["status"] == "tend"
    names = [str(n) for n in z["flx_names"]]
    with netcdf_file(out.flxfile, "r", mmap=False) as nc:
        assert np.array_equal(np.array(nc.variables["kt"][:]), z["his_kt"])
        for q, v in enumerate(names):
            assert np.array_equal(np.array(nc.variables[v][:]).astype(np.float32),
                                  z["flx"][:, q]), v


def test_restart_continues_like_the_oracle(tmp_path):
    """Write a restart mid-run, relaunch a fresh model from it (the warm
    starts are not in the file, as in the reference) and finish the run; the
    oracle does the same from the same file."""
    import torch
    from fluid2d_gb300 import engine
    from oracle import stepper
    z, wl, kw, lk = _fixture("loop_euler_closed_32")
    G = _model(wl, kw, "exact")
    G.loop(lk["tend"], max_steps=12, **_setup_kw(lk))
    path = str(tmp_path / "r.nc")
    G.write_restart(path, lk["tend"])
    H = engine.from_workload(wl, variant="exact", **kw)
    clock = H.read_restart(path)
    assert clock["kt"] == 12
    st = H.loop(clock["tend"], t=clock["t"], kt=clock["kt"], tnexthis=clock["tnexthis"],
                tnextdiag=clock["tnextdiag"], **_setup_kw(lk))
    p, O = stepper.from_workload(wl, **kw)
    from fluid2d_gb300.output import Restart
    _, state = Restart.read(path, O.varname_list)
    O.state[:] = state
    out = stepper.History(lk["var_to_save"], lk["freq_his"], lk["freq_diag"],
                          tnexthis=clock["tnexthis"], tnextdiag=clock["tnextdiag"])
    t, kt, dts, reason = stepper.loop(O, p, clock["tend"], kw["dt"], out, t=clock["t"],
                                      kt=clock["kt"])
    assert st["kt"] == kt and st["t"] == t
    assert [h[1] for h in st["his"]] == [h[1] for h in out.his]
    assert np.array_equal(H.var.state.cpu().numpy(), O.state)
    torch.cuda.synchronize()
