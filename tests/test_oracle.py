"""CPU tests of the oracle (the parity reference), no GPU needed.

* golden: the oracle stepper replays the fixtures of tests/golden/ (made by
  running the reference's own Python over the oracle kernels) bit for bit;
* pin: where the reference sources are present, its Python over the oracle
  kernels equals the oracle stepper (skipped elsewhere);
* invariants of the restated kernels (flux-form conservation, the REAL*4
  reconstruction weights, the 9-point Laplacian of a quadratic, transfer
  operators on constants, V-cycle contraction);
* host logic of the multigrid hierarchy (level sizes).
"""
import ast
import glob
import os

import numpy as np
import pytest

from tests import _cases as C

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
                if not os.path.basename(p).startswith(("loop_", "fluxes_")))


def K():
    from oracle import oracle
    return oracle


def load_golden(path):
    z = np.load(path, allow_pickle=False)
    params = ast.literal_eval(str(z["params"][0]))
    return z, params


def golden_model(path):
    from oracle import stepper
    z, prm = load_golden(path)
    kw = {k: prm[k] for k in ("Rd", "beta", "diffusion", "Kdiff", "noslip",
                                      "hydroepsilon", "order", "flux_splitting_method") if k in prm}
    p = stepper.Param(modelname=prm["model"], nx=prm["nx"], ny=prm["ny"], Lx=prm["Lx"],
                      Ly=prm["Ly"], geometry=prm["geometry"], gravity=prm["gravity"], **kw)
    g = stepper.Grid(p)
    g.msk = z["msk"].copy()
    if "msknoslip" in z:
        g.msknoslip = z["msknoslip"].copy()
    g.finalize_msk()
    M = stepper.MODELS[prm["model"]](p, grid=g)
    if "rhsp" in z:
        M.set_islands(z["rhsp"], z["psi_island"])
    M.state[:] = z["states"][0]
    M.diagnostics()
    return z, p, M


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_golden_replay(path):
    from oracle import stepper
    z, p, M = golden_model(path)
    dt = float(z["dt"])
    states = z["states"]
    t = 0.
    for k in range(1, len(states)):
        t = stepper.run(M, p, 1, dt, t=t)
        assert np.array_equal(M.state, states[k]), (path, k)
        names = [str(n) for n in z["diag_names"]]
        assert [M.diags[n] for n in names] == list(z["diags"][k])


def test_golden_fixtures_exist():
    assert len(GOLDEN) >= 5


def test_reference_python_pin():
    """The reference's Python over the oracle kernels == the oracle stepper."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(HERE, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    from tests.conftest import reference_core
    core = reference_core("operators.py")
    from oracle import stepper
    wl, kw = mg.cases()["euler_closed_32"]
    R = mg.reference_model(core, wl, kw)
    p, O = stepper.from_workload(wl, **kw)
    assert np.array_equal(R.var.state, O.state)


# ---------------------------------------------------------------- invariants
def test_reconstruction_weights_are_real4():
    # 5th-order weights sum to 1.0000000149 (REAL*4 literals, fortran_advection.f90:36-40)
    s = sum(float(np.float32(a) / np.float32(b)) for a, b in
            [(1, 30), (-13, 60), (47, 60), (9, 20), (-1, 20)])
    assert abs(s - 1.0000000149) < 1e-9
    m, n = 22, 40
    msk = np.ones((m, n), dtype=np.int8)
    q = np.full((m, n), 2.0)
    u = np.full((m, n), 0.7)
    v = np.zeros((m, n))
    y = np.zeros((m, n))
    cst = np.array([0.1, 0.1, 0.05, 0.7, 0.05])
    K().adv_upwind(msk, q, y, u, v, cst, 3, 1, 5)
    # uniform flux of a constant field: zero divergence
    assert np.abs(y[3:-3, 3:-3]).max() < 1e-12


@pytest.mark.parametrize("geom,islands", [("closed", 0), ("closed", 3), ("xchannel", 2)])
def test_advection_conserves_the_integral(geom, islands):
    m, n = 38, 54
    msk = C.mask(m, n, geom, islands, 3)
    q, u, v = C.field(m, n, 1) * msk, C.field(m, n, 2), C.field(m, n, 3)
    for a in (q, u, v):  # fields consistent with the periodic direction
        K().fillhalo(a, 3)
    y = np.zeros((m, n))
    K().adv_upwind(msk, q, y, u, v, np.array([0.1, 0.1, 0.05, 1.0, 0.05]), 3, 1, 5)
    # telescoping fluxes: walls carry no flux, periodic ends cancel
    assert abs(y[3:-3, 3:-3].sum()) < 1e-9 * np.abs(y).sum()


def test_laplacian_of_a_quadratic():
    from tests.test_gpu_kernels import _hierarchy
    L0 = _hierarchy(38, 38, "perio", 0, 1)[0]
    m, n = L0.mv, L0.nv
    h = L0.dx
    jj, ii = np.meshgrid(np.arange(m) * h, np.arange(n) * h, indexing="ij")
    x = 0.5 * (ii ** 2 + jj ** 2)
    b = np.zeros((m, n))
    r = np.zeros((m, n))
    K().computeresidualwitha(L0.msk, L0.A[:, :, :5], x, b, r)
    inner = (slice(4, -4), slice(4, -4))
    fluid = L0.msk[inner] != 0
    # A x = lap(x) = 2 exactly for a quadratic (9-point stencil): r = -2
    np.testing.assert_allclose(r[inner][fluid], -2.0, rtol=1e-9)


def test_transfer_operators_on_constants():
    from tests.test_gpu_kernels import _hierarchy
    levs = _hierarchy(70, 70, "perio", 0, 2)
    f, c = levs[0], levs[1]
    x1 = np.full((f.mv, f.nv), 3.0)
    x2 = np.zeros((c.mv, c.nv))
    K().restrict(c.msk, x1, 3, x2)
    assert np.allclose(x2[3:-3, 3:-3][c.msk[3:-3, 3:-3] != 0], 3.0)
    y1 = np.zeros((f.mv, f.nv))
    K().interpolate(f.msk, c.msk, np.full((c.mv, c.nv), 2.0), 3, y1)
    inner = (slice(3, -4), slice(3, -4))
    assert np.allclose(y1[inner][f.msk[inner] != 0], 2.0)


def test_vcycle_contracts_the_residual():
    from oracle import stepper
    msk = C.corner_mask(C.mask(70, 70, "closed", 2, 4))
    pp = {'nh': 3, 'n': 64, 'm': 64, 'omega': 8. / 9., 'dx': 1. / 64, 'dy': 1. / 64}
    G = stepper.Gmg(pp, msk * 1.)
    b = C.field(70, 70, 5) * (msk != 0)
    x = np.zeros((70, 70))
    g0 = G.grid[0]
    r = np.zeros_like(x)
    g0.residual(x, b, r)
    n0 = g0.norm(r)
    G.twoVcycle(x, b)
    g0.residual(x, b, r)
    assert g0.norm(r) < 0.1 * n0


# ---------------------------------------------------------------- host logic
@pytest.mark.parametrize("n,m,levels,coarsest", [
    (1024, 1024, 9, (4, 4)), (2048, 512, 8, (16, 4)), (128, 128, 6, (4, 4)),
    (320, 192, 7, (5, 3)), (64, 640, 5, (4, 40))])
def test_gridinfo_levels(n, m, levels, coarsest):
    from oracle import stepper
    info = stepper.gridinfo(n, m, 1. / n, 1. / n)
    assert len(info) == levels
    assert (info[-1]["n"], info[-1]["m"]) == coarsest
