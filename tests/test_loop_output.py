"""CPU tests of the time loop and of the history / diagnostic / restart files.

* the oracle's Fluid2d.loop restatement replays the loop fixtures of
  tests/golden/ (made by running the reference's own Fluid2d.loop and Output
  over the oracle kernels) bit for bit: dt sequence, record times and
  iterations, float32 history planes, diagnostic rows, final state;
* where the reference sources are present: the reference loop still equals
  the fixture, and the reference's NcfileIO / create_diag / Restart.write
  (through an in-memory netCDF recorder) produce the variables, types,
  shapes, values and attributes that fluid2d_gb300.output writes;
* the writers round-trip.
"""
import ast
import glob
import importlib.util
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
LOOPS = sorted(glob.glob(os.path.join(HERE, "golden", "loop_*.npz")))


def make_golden():
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def reference_core():
    from tests.conftest import reference_core as core
    return core()


def load_loop(path):
    z = np.load(path, allow_pickle=False)
    prm = ast.literal_eval(str(z["params"][0]))
    lk = ast.literal_eval(str(z["loop"][0]))
    return z, prm, lk


def fixture_workload(name):
    """The workload a loop fixture was made from (same generator, same seed)."""
    mg = make_golden()
    mk, kw, lk = mg.LOOP_CASES[name]
    return mk(), kw, lk


@pytest.mark.parametrize("path", LOOPS, ids=[os.path.basename(p) for p in LOOPS])
def test_loop_golden_replay(path):
    from oracle import stepper
    name = os.path.basename(path)[:-4]
    z, prm, lk = load_loop(path)
    wl, kw, lk2 = fixture_workload(name)
    assert lk == lk2
    assert np.array_equal(wl["msk"], z["msk"])
    p, O = stepper.from_workload(wl, **kw)
    O.state[:] = z["init_state"]
    fl = stepper.Fluxes(O) if lk.get("diag_fluxes") else None
    out = stepper.History(lk["var_to_save"], lk["freq_his"], lk["freq_diag"], fluxes=fl)
    t, kt, dts, reason = stepper.loop(O, p, lk["tend"], kw["dt"], out,
                                      exacthistime=lk["exacthistime"],
                                      rescaledtime=lk.get("rescaledtime", "none"))
    assert reason == "tend"
    assert np.array_equal(np.array(dts), z["dts"])
    assert np.array_equal(np.array([h[0] for h in out.his]), z["his_t64"])
    assert np.array_equal(np.array([h[0] for h in out.his], np.float32), z["his_t"])
    assert np.array_equal(np.array([h[1] for h in out.his], np.int32), z["his_kt"])
    for v in lk["var_to_save"]:
        assert np.array_equal(np.array([h[2][v] for h in out.his]), z["his_" + v]), v
    names = [str(n) for n in z["diag_names"]]
    assert np.array_equal(np.array([[d[2][k] for k in names] for d in out.diag]), z["diag64"])
    assert np.array_equal(O.state, z["final_state"])
    if fl is not None:
        assert [str(n) for n in z["flx_names"]] == fl.fullflx_list
        assert np.array_equal(np.array([[f[2][v] for v in fl.fullflx_list] for f in out.flx]),
                              z["flx"])


def test_loop_fixtures_exist():
    assert len(LOOPS) >= 4


def test_exacthistime_lands_on_history_times():
    z, prm, lk = load_loop(os.path.join(HERE, "golden", "loop_euler_closed_32.npz"))
    want = lk["freq_his"] * np.arange(len(z["his_t64"]))
    assert np.allclose(z["his_t64"], want, rtol=0, atol=1e-15)
    # the countdown shrinks dt over the 8 steps before each history time
    dts = z["dts"]
    assert dts[7] < dts[6] < dts[0]


def test_reference_loop_pin():
    """The reference's own Fluid2d.loop + Output still give the fixture."""
    import tempfile
    core = reference_core()
    mg = make_golden()
    from oracle import refshim
    refshim.install(core)
    path = os.path.join(HERE, "golden", "loop_euler_closed_32.npz")
    z, prm, lk = load_loop(path)
    mk, kw, _ = mg.LOOP_CASES["loop_euler_closed_32"]
    with tempfile.TemporaryDirectory() as tmp:
        R, his, dia, init = mg.reference_loop(core, mk(), kw, lk, tmp)
    assert np.array_equal(init, z["init_state"])
    assert np.array_equal(his["t"], z["his_t"])
    assert np.array_equal(his["kt"], z["his_kt"])
    for v in lk["var_to_save"]:
        assert np.array_equal(his[v], z["his_" + v])
    assert np.array_equal(R.var.state, z["final_state"])


# ---------------------------------------------------------------- writers
def _read(path):
    from scipy.io import netcdf_file
    with netcdf_file(path, "r", mmap=False) as nc:
        return ({k: (v.typecode(), v.dimensions,
                     np.array(v[:]).astype(v[:].dtype.newbyteorder("=")))
                 for k, v in nc.variables.items()},
                dict(nc._attributes), {k: nc.dimensions[k] for k in nc.dimensions})


def _grid(nx=12, ny=8, geometry="closed"):
    from fluid2d_gb300 import workloads as W
    return W.base_mask(nx, ny, geometry)


def test_history_and_diag_roundtrip(tmp_path):
    from fluid2d_gb300.output import Output
    msk = _grid()
    out = Output(str(tmp_path), "exp", ["vorticity", "psi"], msk, 1.5, 1.0,
                 param={"nx": 12, "ny": 8, "adaptable_dt": True, "expname": "exp",
                        "tracer_list": ["vorticity"]})
    rng = np.random.default_rng(0)
    recs = []
    for k in range(3):
        f = {"vorticity": rng.standard_normal((8, 12)), "psi": rng.standard_normal((14, 18))}
        out.write_his(0.1 * k, 4 * k, f)
        recs.append(f)
    for k in range(4):
        out.write_diag(0.05 * k, 2 * k, {"maxspeed": 1. + k, "ke": 0.5 * k})
    var, att, dims = _read(out.hisfile)
    assert dims == {"t": None, "x": 12, "y": 8}
    assert var["vorticity"][0] == "f" and var["vorticity"][1] == ("t", "y", "x")
    assert var["kt"][0] == "i" and var["msk"][0] == "i"
    assert np.array_equal(var["vorticity"][2], np.array([r["vorticity"] for r in recs],
                                                        np.float32))
    assert np.array_equal(var["psi"][2], np.array([r["psi"][3:-3, 3:-3] for r in recs],
                                                  np.float32))
    assert np.array_equal(var["kt"][2], [0, 4, 8])
    assert np.allclose(var["x"][2], (np.arange(12) + 0.5) * 1.5 / 12)
    assert np.array_equal(var["msk"][2], msk[3:-3, 3:-3])
    assert att["adaptable_dt"] == 1 and "tracer_list" not in att
    dvar, _, _ = _read(out.diagfile)
    assert np.array_equal(dvar["maxspeed"][2], np.array([1., 2., 3., 4.], np.float32))
    assert np.array_equal(dvar["kt"][2], [0, 2, 4, 6])


def test_restart_roundtrip(tmp_path):
    from fluid2d_gb300.output import Restart
    names = ["vorticity", "psi", "u", "v", "source"]
    state = np.random.default_rng(1).standard_normal((5, 14, 18))
    rs = Restart(str(tmp_path), "exp")
    assert rs.last() is None
    path = rs.path(0)
    Restart.write(path, 2.0, 0.75, 0.01, 75, 0.8, 1.0, state, names)
    assert rs.last() == 0
    clock, st = Restart.read(path, names)
    assert clock == {"tend": 2.0, "t": 0.75, "dt": 0.01, "kt": 75, "tnextdiag": 0.8,
                     "tnexthis": 1.0}
    assert np.array_equal(st, state)


def test_writers_match_reference_layout(tmp_path):
    """The reference's NcfileIO.create/write, create_diag and Restart.write,
    run through the in-memory netCDF recorder, against these writers."""
    import contextlib
    import io
    import types
    core = reference_core()
    from oracle import refshim
    from fluid2d_gb300.output import NcfileIO, Output, Restart, cell_centres, _attrs_of
    p = refshim.reference_param(core, nx=16, ny=8, Lx=2., Ly=1., geometry="closed")
    rec = refshim.install_recording_netcdf()
    import grid as rgrid
    import output as routput
    import restart as rrestart
    routput.Dataset = rrestart.Dataset = rec
    with contextlib.redirect_stdout(io.StringIO()):
        g = rgrid.Grid(p)
    p.varname_list = ["vorticity", "psi", "u", "v", "source"]
    rng = np.random.default_rng(2)
    state = rng.standard_normal((5, 14, 22))
    ref = routput.NcfileIO(p, g, "ref_his", ["vorticity", "psi"], p.varname_list)
    ref.create()
    ref.write(state, 0.25, 7)
    ref.write(state * 2, 0.5, 14)
    mine = NcfileIO(str(tmp_path / "his.nc"), ["vorticity", "psi"], g.msk,
                    cell_centres(16, 2.), cell_centres(8, 1.), _attrs_of(p))
    mine.create()
    mine.write({"vorticity": state[0], "psi": state[1]}, 0.25, 7)
    mine.write({"vorticity": 2 * state[0], "psi": 2 * state[1]}, 0.5, 14)
    R = rec.FILES["ref_his"]
    var, att, dims = _read(mine.ncfile)
    assert R["dims"] == dims
    assert set(R["variables"]) == set(var)
    for k, v in R["variables"].items():
        assert v.a.dtype == var[k][2].dtype, k
        assert np.array_equal(v.a, var[k][2]), k
    for k, v in R["attrs"].items():
        assert k in att, k
        a = att[k].decode() if isinstance(att[k], bytes) else att[k]
        assert a == v or np.isclose(a, v), k

    # diagnostic file
    o = types.SimpleNamespace(diagfile="ref_diag", list_diag=["maxspeed", "ke"])
    routput.Output.create_diag(o, None)
    mo = Output(str(tmp_path), "m", ["vorticity"], g.msk, 2., 1.)
    mo.create_diag(["maxspeed", "ke"])
    dvar, _, _ = _read(mo.diagfile)
    D = rec.FILES["ref_diag"]
    assert set(D["variables"]) == set(dvar)
    for k, v in D["variables"].items():
        assert v.a.dtype == dvar[k][2].dtype, k

    # restart file
    var_obj = types.SimpleNamespace(get=lambda v: state[p.varname_list.index(v)])
    rs = types.SimpleNamespace(restart_file="ref_restart", nxl=22, nyl=14,
                               varname_list=p.varname_list)
    rrestart.Restart.write(rs, 3., 1.25, 0.01, 125, 1.3, 1.5, var_obj)
    path = str(tmp_path / "r.nc")
    Restart.write(path, 3., 1.25, 0.01, 125, 1.3, 1.5, state, p.varname_list)
    RR = rec.FILES["ref_restart"]
    rvar, ratt, rdims = _read(path)
    assert RR["dims"] == rdims
    for k, v in RR["variables"].items():
        assert v.a.dtype == rvar[k][2].dtype == np.float64
        assert np.array_equal(v.a, rvar[k][2])
    for k, v in RR["attrs"].items():
        assert ratt[k] == v, k


def test_island_arrays_match_reference_fixture():
    """fluid2d_gb300.island (host restatement of core/island.py) gives the
    rhsp and psi arrays the reference's Island computed for the fixture."""
    from fluid2d_gb300.island import Island
    mg = make_golden()
    z = np.load(os.path.join(HERE, "golden", "euler_xchannel_64x32_islands_noslip.npz"))
    wl = mg.channel_with_islands()
    I = Island(wl["nx"] + 6, wl["ny"] + 6, wl["Lx"] / wl["nx"], wl["Ly"] / wl["ny"])
    for idx, psi0 in wl["islands"]:
        I.add(idx, psi0)
    rhsp, psi = I.finalize()
    assert np.array_equal(rhsp, z["rhsp"]) and np.array_equal(psi, z["psi_island"])
    assert np.array_equal(wl["msknoslip"], z["msknoslip"])
