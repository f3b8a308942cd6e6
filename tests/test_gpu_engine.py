"""Step-level parity of the device engine against the oracle stepper.

With the exact build, closed-domain Euler, Boussinesq and QG states after
several RK3 steps are bit-identical to the oracle (the only reductions that
feed the state are maxima); the periodic Euler case differs by the rounding
of the mean of psi (a sum), so it is compared with a tolerance.  The product
build (FMA contraction) is compared at 1e-10 relative L-inf, the parity bar
after 10 steps.
"""
import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import torch
    from fluid2d_gb300 import engine
    assert torch.cuda.is_available()
    return engine


def relerr(a, b):
    return np.abs(a - b).max() / max(1e-300, np.abs(b).max())


def _workloads():
    from fluid2d_gb300 import workloads as W
    qg = W.dipole(64, 64, seed=7)
    qg["model"] = "quasigeostrophic"
    qg["fields"] = {"pv": qg["fields"]["vorticity"]}
    isl = W.dipole(64, 48, seed=9)
    isl["msk"] = C.mask(54, 70, "closed", 2, 9)
    isl["fields"]["vorticity"] = isl["fields"]["vorticity"] * isl["msk"]
    return {
        "euler-closed-dipole": W.dipole(64, 64),
        "euler-closed-islands": isl,
        "euler-perio-turb": W.turbulence(64, 64, seed=5),
        "boussinesq-xchannel": W.shear(128, 32, seed=3),
        "qg-closed": qg,
    }


WL = list(_workloads().keys())


def _pair(eng, name, variant, steps):
    import torch
    wl = _workloads()[name]
    kw = {"Rd": 0.3, "beta": 2.0} if wl["model"] == "quasigeostrophic" else {}
    p, O = C.oracle_model(wl, **kw)
    dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
    G = eng.from_workload(wl, variant=variant, dt=dt, **kw)
    if wl["model"] == "quasigeostrophic":
        G.get("pv").copy_(torch.from_numpy(O.get("pv")).cuda())
    G.set_psi_from_vorticity()
    G.diagnostics()
    s0 = G.var.state.cpu().numpy()
    from oracle import stepper
    stepper.run(O, p, steps, dt)
    G.run(steps)
    torch.cuda.synchronize()
    return O, G, s0


@pytest.mark.parametrize("name", WL)
def test_initial_solve(eng, name):
    import torch
    wl = _workloads()[name]
    kw = {"Rd": 0.3, "beta": 2.0} if wl["model"] == "quasigeostrophic" else {}
    p, O = C.oracle_model(wl, **kw)
    G = eng.from_workload(wl, variant="exact", **kw)
    if wl["model"] == "quasigeostrophic":
        G.get("pv").copy_(torch.from_numpy(O.get("pv")).cuda())
    G.set_psi_from_vorticity()
    d = G.diagnostics()
    st = G.var.state.cpu().numpy()
    tol = 1e-13 if wl["geometry"] == "perio" else 0.
    for k, nm in enumerate(G.var.varname_list):
        assert relerr(st[k], O.state[k]) <= tol, (nm, relerr(st[k], O.state[k]))
    assert d["maxspeed"] == O.diags["maxspeed"] or tol
    assert G.solve_stats()[0] == O.ope.last_solve[0]


@pytest.mark.parametrize("variant", ["exact", "product"])
@pytest.mark.parametrize("name", WL)
def test_steps(eng, name, variant):
    steps = 5
    O, G, _ = _pair(eng, name, variant, steps)
    st = G.var.state.cpu().numpy()
    d = G.read_diags()
    exact = variant == "exact" and "perio" not in name
    for k, nm in enumerate(G.var.varname_list):
        e = relerr(st[k], O.state[k])
        if exact:
            assert np.array_equal(st[k], O.state[k]), (nm, e)
        else:
            assert e <= 1e-10, (nm, e)
    for k, v in d.items():
        assert abs(v - O.diags[k]) <= 1e-9 * max(1e-12, abs(O.diags[k])) + 1e-300 or \
            abs(v - O.diags[k]) < 1e-14, (k, v, O.diags[k])


@pytest.mark.parametrize("name", ["euler-closed-dipole", "boussinesq-xchannel"])
def test_graph_replay_matches_eager(eng, name):
    import torch
    wl = _workloads()[name]
    A = eng.from_workload(wl, variant="product", dt=1e-3)
    B = eng.from_workload(wl, variant="product", dt=1e-3)
    for M in (A, B):
        M.set_psi_from_vorticity()
        M.diagnostics()
    A.run(4)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        B.run(4, graph=True)
    s.synchronize()
    torch.cuda.synchronize()
    assert torch.equal(A.var.state, B.var.state)


def test_run_host_equals_the_device_steps(eng):
    """Model.run_host (the state uploaded from page-locked host memory,
    stepped and read back every step, one captured graph) gives the device
    path's state bit for bit, in the host buffer and on the device."""
    import torch
    wl = _workloads()["euler-perio-turb"]
    A = eng.from_workload(wl, variant="product", dt=1e-3)
    B = eng.from_workload(wl, variant="product", dt=1e-3)
    for M in (A, B):
        M.set_psi_from_vorticity()
        M.diagnostics()
    host = torch.empty(B.var.state.shape, dtype=torch.float64).pin_memory()
    host.copy_(B.var.state.cpu())
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        A.run(3, graph=True)
        B.run_host(3, host)
    s.synchronize()
    assert torch.equal(A.var.state.cpu(), host)
    assert torch.equal(A.var.state, B.var.state)
    with pytest.raises(ValueError):
        B.run_host(1, torch.zeros(B.var.state.shape, dtype=torch.float64))


def test_gmg_twovcycle_and_solve(eng):
    import torch
    from oracle import stepper
    for (m, n, geom, isl, seed) in [(70, 70, "closed", 2, 1), (38, 134, "perio", 0, 2),
                                   (134, 70, "xchannel", 3, 3)]:
        msk = C.corner_mask(C.mask(m, n, geom, isl, seed))
        dx = 1. / (n - 6)
        pp = {'nh': 3, 'n': n - 6, 'm': m - 6, 'omega': 8. / 9., 'dx': dx, 'dy': dx}
        O = stepper.Gmg(pp, msk * 1.)
        G = eng.Gmg(msk, n - 6, m - 6, dx, dx, variant="exact")
        x, b = C.field(m, n, seed), C.field(m, n, seed + 1)
        xo = x.copy()
        O.twoVcycle(xo, b)
        xg = torch.from_numpy(x).cuda()
        G.twoVcycle(xg, torch.from_numpy(b).cuda())
        assert np.array_equal(xg.cpu().numpy(), xo), relerr(xg.cpu().numpy(), xo)
        xo = x.copy()
        nite_o, res_o = O.solve(xo, b, {'maxite': 4, 'tol': 1e-11})
        xg = torch.from_numpy(x).cuda()
        nite_g, res_g = G.solve(xg, torch.from_numpy(b).cuda())
        assert nite_g == nite_o
        assert abs(res_g - res_o) <= 1e-6 * res_o
        assert np.array_equal(xg.cpu().numpy(), xo), relerr(xg.cpu().numpy(), xo)


@pytest.mark.parametrize("geom,hyd,dyfac", [("xchannel", 0.1, 1.), ("closed", 0.1, 1.),
                                            ("xchannel", 1., 1. / 6), ("perio", 1., 1. / 6)])
def test_gmg_line_relaxation(eng, geom, hyd, dyfac):
    """Hierarchies relaxed by smoothtridiag (hydroepsilon*dy/dx <= 0.2): the
    device twoVcycle and solve equal the oracle's bit for bit (exact build);
    the periodic solve differs only by the rounding of its norms."""
    import torch
    from oracle import stepper
    m, n = 22, 70
    msk = C.corner_mask(C.mask(m, n, geom, 0, 1))
    dx = 4. / (n - 6)
    dy = dx * dyfac
    pp = {'nh': 3, 'n': n - 6, 'm': m - 6, 'omega': 8. / 9., 'dx': dx, 'dy': dy,
          'hydroepsilon': hyd}
    O = stepper.Gmg(pp, msk * 1.)
    assert all(L.relaxation == 'tridiagonal' for L in O.grid)
    G = eng.Gmg(msk, n - 6, m - 6, dx, dy, hydroepsilon=hyd, variant="exact")
    x, b = C.field(m, n, 1), C.field(m, n, 2)
    xo = x.copy()
    O.twoVcycle(xo, b)
    xg = torch.from_numpy(x).cuda()
    G.twoVcycle(xg, torch.from_numpy(b).cuda())
    assert np.array_equal(xg.cpu().numpy(), xo)
    xo = x.copy()
    O.solve(xo, b, {'maxite': 4, 'tol': 1e-11})
    xg = torch.from_numpy(x).cuda()
    G.solve(xg, torch.from_numpy(b).cuda())
    assert relerr(xg.cpu().numpy(), xo) <= 1e-13


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coarse_level_changes_nothing_but_launches(eng, precision):
    """Any switch level of the single-CTA coarse solve gives the same state
    bit for bit (exact build), and the autotuner picks one of them."""
    import torch
    from fluid2d_gb300 import workloads as W
    from fluid2d_gb300.autotune import tune_coarse_level
    wl = W.dipole(128, 96, seed=3)
    states = []
    probe = eng.from_workload(wl, variant="exact", precision=precision, dt=2e-3)
    cur, first, nlev = probe.coarse_switch()
    assert first <= cur <= nlev
    for level in sorted({first, (first + nlev) // 2, nlev}):
        M = eng.from_workload(wl, variant="exact", precision=precision, dt=2e-3)
        M.set_psi_from_vorticity()
        M.diagnostics()
        M.coarse_switch(level)
        M.run(3)
        torch.cuda.synchronize()
        states.append(M.var.state.clone())
    for st in states[1:]:
        assert torch.equal(st, states[0])
    M = eng.from_workload(wl, precision=precision, dt=2e-3)
    M.set_psi_from_vorticity()
    M.diagnostics()
    best, times = tune_coarse_level(M, steps=2, warmup=1, use_cache=False)
    assert best in times and M.coarse_switch()[0] == best


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["euler-perio-turb", "euler-closed-dipole", "boussinesq-xchannel"])
def test_coarse_operator_matches_the_cycle(eng, name, precision):
    """The product build applies the coarse part of the cycles started from
    x = 0 as its precomputed linear map: the same function summed in another
    order.  Its states differ from the cycle-by-cycle path by no more than
    the product build's own FMA contraction moves them away from the exact
    build (an order of magnitude of slack), at every switch level.  The exact
    build never builds it."""
    import torch
    wl = _workloads()[name]

    def run(variant, level, op):
        M = eng.from_workload(wl, variant=variant, precision=precision, dt=1e-3)
        M.coarse_switch(level)
        n = M.coarse_operator(op) if variant == "product" else M.coarse_operator()
        M.set_psi_from_vorticity()
        M.diagnostics()
        M.run(4)
        torch.cuda.synchronize()
        return M.var.state.cpu().numpy(), n

    probe = eng.from_workload(wl, precision=precision, dt=1e-3)
    cur, first, nlev = probe.coarse_switch()
    for level in sorted({first, nlev - 1}):
        ex, n_ex = run("exact", level, None)
        assert n_ex == 0
        on, n_on = run("product", level, True)
        off, n_off = run("product", level, False)
        assert n_on > 0 and n_off == 0
        for k in range(on.shape[0]):
            fma = relerr(off[k], ex[k])
            assert relerr(on[k], off[k]) <= max(1e-12, 10 * fma), (level, k, fma)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["euler-perio-turb", "euler-closed-dipole", "euler-islands-square",
                                  "boussinesq-xchannel", "qg-closed", "euler-closed-islands",
                                  "euler-closed-5point"])
def test_column_sweeps_match_the_sweep_kernels(eng, name, precision):
    """The float64 sweeps and residual in column form (four points a thread,
    neighbourhoods in registers; on the finest level fluid 3x3 blocks go
    through the separable form of the 9-point operator, on the stored levels
    points with the level's uniform stencil through its row-sum form)
    compute the reference's function in another order of operations: the
    states after four steps agree with the sweep, residual and fused level
    kernels (reference order) to the product build's rounding, on periodic
    and closed domains, islands, the Helmholtz operator of QG and 5-point
    finest operators (dx != dy: there only the stored levels change); in the
    mixed form the float64 defect's residual and the float stored levels
    take the column form.  Mode 2
    forces the column form on these grids of fewer CTAs than SMs (ragged
    last columns of threads and of rows); a replayed graph gives the eager
    steps' bits."""
    import torch
    from fluid2d_gb300 import _lib
    from fluid2d_gb300 import workloads as W
    wls = dict(_workloads())
    wls["euler-closed-5point"] = W.dipole(64, 48, seed=2)
    # the islands workload with dx = dy: the 9-point operator, and points
    # whose 3x3 blocks touch an island take the general expression
    wls["euler-islands-square"] = dict(wls["euler-closed-islands"], Ly=0.75)
    five_point = ("euler-closed-islands", "euler-closed-5point")
    wl = wls[name]
    P = _lib.lib("product")

    def run(mode, graph=False):
        old = P.f2d_set_separable(mode)
        try:
            kw = {"Rd": 0.3, "beta": 2.0} if wl["model"] == "quasigeostrophic" else {}
            M = eng.from_workload(wl, dt=1e-3, precision=precision, **kw)
            M.set_psi_from_vorticity()
            M.diagnostics()
            if graph:
                s = torch.cuda.Stream()
                with torch.cuda.stream(s):
                    M.run(4, graph=True)
                s.synchronize()
            else:
                M.run(4)
            torch.cuda.synchronize()
            return M.var.state.cpu().numpy()
        finally:
            P.f2d_set_separable(old)

    assert P.f2d_set_separable(-1) == 1
    a, b, g = run(2), run(0), run(2, graph=True)
    # u and v (planes 2 and 3 of every model) against the velocity's scale:
    # v is ~0 in the parallel shear flow
    vel = max(np.abs(b[2]).max(), np.abs(b[3]).max())
    tol = 1e-12 if precision == "fp64" else 1e-6
    for k in range(a.shape[0]):
        scale = vel if k in (2, 3) else max(np.abs(b[k]).max(), 1e-300)
        assert np.abs(a[k] - b[k]).max() <= tol * scale, k
        assert np.array_equal(a[k], g[k]), k
    # the column forms ran (the mixed form's float32 cycles may round both
    # residuals to the same floats); with dx != dy the finest operator is
    # the 5-point one and the coarsened ones carry rounding noise from point
    # to point (no uniform stencil): the reference kernels run everywhere
    if precision == "fp64":
        assert np.array_equal(a, b) == (name in five_point)
    assert _lib.lib("exact").f2d_set_separable(-1) == 0


@pytest.mark.parametrize("geom,islands", [("perio", 0), ("closed", 3), ("xchannel", 2)])
def test_stored_level_column_sweeps(eng, geom, islands):
    """A V-cycle from level 1 (no finest-level kernel) with the stored
    levels' column-form sweeps (points with the level's uniform stencil in
    row-sum form, the others in the reference's expression) against the
    fused level smoother: the same function to the product build's rounding,
    not the same bits (the column form ran), on periodic, closed and channel
    masks with islands."""
    import torch
    from fluid2d_gb300 import _lib
    P = _lib.lib("product")
    n = 256
    msk = C.corner_mask(C.mask(n + 6, n + 6, geom, islands, 4))
    dx = 1. / n

    def vcycle(mode):
        old = P.f2d_set_separable(mode)
        try:
            G = eng.Gmg(msk, n, n, dx, dx, variant="product")
            mv, nv = G.shapes[1]
            G.level_array(1, "x").copy_(torch.from_numpy(C.field(mv, nv, 5)).cuda())
            G.level_array(1, "b").copy_(torch.from_numpy(C.field(mv, nv, 6, scale=1e5)).cuda())
            G.Vcycle(1)
            torch.cuda.synchronize()
            return G.level_array(1, "x").cpu().numpy()
        finally:
            P.f2d_set_separable(old)

    a, b = vcycle(2), vcycle(0)
    assert relerr(a, b) <= 1e-12
    assert not np.array_equal(a, b)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_l2_persisting_windows_change_nothing_but_timing(eng, precision):
    """The persisting L2 access-policy windows on the multigrid cycles'
    launches (f2d_set_l2_persist) leave every state bit unchanged, eager and
    replayed from a graph."""
    import torch
    from fluid2d_gb300 import _lib
    from fluid2d_gb300 import workloads as W
    P = _lib.lib("product")
    wl = W.turbulence(256, 256, seed=3)

    def run(mode):
        old = P.f2d_set_l2_persist(mode)
        try:
            M = eng.from_workload(wl, dt=1e-3, precision=precision)
            M.set_psi_from_vorticity()
            M.diagnostics()
            M.run(2)
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())  # the eager steps first
            with torch.cuda.stream(s):
                M.run(2, graph=True)
            s.synchronize()
            return M.var.state.cpu().numpy()
        finally:
            P.f2d_set_l2_persist(old)

    assert P.f2d_set_l2_persist(-1) == 1
    assert np.array_equal(run(1), run(0))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_level_tiles_change_nothing_but_launches(eng, precision):
    """Every CTA tile target and smoother block size of the level kernels
    gives the same state bit for bit (exact build); the tuner keeps one."""
    import torch
    from fluid2d_gb300 import _lib, workloads as W
    from fluid2d_gb300.autotune import tune_level_tiles
    L = _lib.lib("exact")
    prev = (L.f2d_set_level_tiles(-2), L.f2d_set_level_threads(-1))
    wl = W.dipole(160, 96, seed=5)
    states = []
    try:
        for target, threads in ((0, 0), (64, 0), (1000, 0), (0, 1), (0, 2), (500, 2)):
            L.f2d_set_level_tiles(target)
            L.f2d_set_level_threads(threads)
            M = eng.from_workload(wl, variant="exact", precision=precision, dt=2e-3)
            M.set_psi_from_vorticity()
            M.diagnostics()
            M.run(3)
            torch.cuda.synchronize()
            states.append(M.var.state.clone())
    finally:
        L.f2d_set_level_tiles(prev[0])
        L.f2d_set_level_threads(prev[1])
    for st in states[1:]:
        assert torch.equal(st, states[0])
    M = eng.from_workload(wl, precision=precision, dt=2e-3)
    M.set_psi_from_vorticity()
    M.diagnostics()
    best, times = tune_level_tiles(M, steps=2, warmup=1, use_cache=False)
    assert best in times and len(times) >= 2
    P = _lib.lib("product")
    P.f2d_set_level_tiles(0)
    P.f2d_set_level_threads(0)


def test_fp64_peak_and_profile_step(eng, capsys):
    """The live float64 FMA peak is a plausible figure for this part, and
    bench.py's profiling mode runs an NVTX-bracketed step (single model and
    batched ensemble)."""
    import ctypes
    import bench
    from fluid2d_gb300 import _lib
    v = ctypes.c_double()
    assert _lib.lib().f2d_fp64_peak(ctypes.byref(v)) == 0
    assert 0.05 < v.value < 100., v.value
    bench.profile_step(["--n", "64", "--coarse-level", "3"])
    bench.profile_step(["--n", "64", "--precision", "mixed", "--no-coarse-operator"])
    bench.profile_step(["--ensemble", "3", "--precision", "mixed", "--groups", "2",
                        "--coarse-offset", "1", "--balanced"])
    out = capsys.readouterr().out
    assert "coarse operator 0 points" in out and "batched launches per step" in out
