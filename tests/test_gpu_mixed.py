"""The mixed-precision form against the float64 oracle.

Fluxes in float32, multigrid cycles in float32 inside a float64 defect
correction (float64 residual and psi accumulation), float64 RK accumulation
and diagnostics.  Bar: single-step relative L2 error <= 1e-6
per field against the float64 oracle from an identical state.
"""
import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return np.sqrt(((a - b) ** 2).sum()) / max(1e-300, np.sqrt((b ** 2).sum()))


def _workloads():
    from fluid2d_gb300 import workloads as W
    qg = W.dipole(64, 64, seed=7)
    qg["model"] = "quasigeostrophic"
    qg["fields"] = {"pv": qg["fields"]["vorticity"]}
    return {
        "euler-closed-dipole-128": (W.dipole(128, 128), {}),
        "euler-perio-turb-128": (W.turbulence(128, 128, seed=5), {}),
        "boussinesq-shear-128x32": (W.shear(128, 32, seed=3, delta=0.05), {}),
        "qg-closed-64": (qg, {"Rd": 0.3, "beta": 2.0}),
        "euler-islands-96x64": (C.island_workload(), {}),
    }


@pytest.mark.parametrize("name", list(_workloads().keys()))
def test_mixed_single_and_multi_step_error(name):
    import torch
    from fluid2d_gb300 import engine
    from oracle import stepper
    wl, kw = _workloads()[name]
    p, O = stepper.from_workload(wl, **kw)
    dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
    G = engine.from_workload(wl, precision="mixed", dt=dt, **kw)
    G.var.state.copy_(torch.from_numpy(O.state).cuda())  # identical state
    G.diagnostics()
    errs = []
    names = G.var.varname_list
    for k in range(10):
        stepper.run(O, p, 1, dt)
        G.run(1)
        st = G.var.state.cpu().numpy()
        e = {nm: rel_l2(st[i], O.state[i]) for i, nm in enumerate(names)
             if np.abs(O.state[i]).max() > 0 and nm not in ("u", "v")}
        # velocity components relative to the velocity vector's norm (a
        # component can be ~0, e.g. v in a parallel shear flow)
        iu, iv = names.index("u"), names.index("v")
        nrm = np.sqrt((O.state[iu] ** 2).sum() + (O.state[iv] ** 2).sum())
        e["velocity"] = np.sqrt(((st[iu] - O.state[iu]) ** 2).sum()
                                + ((st[iv] - O.state[iv]) ** 2).sum()) / nrm
        errs.append(e)
    for nm, e in errs[0].items():
        assert e <= 1e-6, (name, "step 1", nm, e)
    for nm, e in errs[-1].items():
        assert e <= 1e-5, (name, "step 10", nm, e)
    nite, res, st = G.solve_stats()
    if wl["model"] != "boussinesq":
        assert st == 0 and nite <= 4 and res < 1e-8


@pytest.mark.parametrize("levels", [8, 1])
@pytest.mark.parametrize("name", ["turbulence-256", "islands-256", "shear-512x128", "qg-256"])
def test_cluster_subcycle_equals_the_level_kernels(name, levels):
    """Mixed form, product build: the small levels' V- and F-cycles as one
    launch of a 16-CTA cluster (levels in distributed shared memory, ghost
    rows exchanged between phases) evaluate the level kernels' expressions
    in their order: the states after three steps equal the level kernels'
    bit for bit, on periodic, closed-with-islands and channel domains and
    QG's Helmholtz operator, with every level that fits in the cluster or
    only the one above the coarse operator's.  Both run the level kernels in
    the reference's order (f2d_set_separable 0: no column or uniform-stencil
    forms), which the cluster reproduces."""
    import torch
    from fluid2d_gb300 import _lib, engine
    from fluid2d_gb300 import workloads as W
    if name == "turbulence-256":
        wl = W.turbulence(256, 256, seed=11)
    elif name == "shear-512x128":
        wl = W.shear(512, 128, seed=12)
    else:
        wl = W.dipole(256, 256, seed=13)
        if name == "islands-256":
            from tests import _cases as C
            wl["msk"] = C.mask(262, 262, "closed", 4, 13)
            wl["fields"]["vorticity"] = wl["fields"]["vorticity"] * wl["msk"]
        else:
            wl["model"] = "quasigeostrophic"
            wl["fields"] = {"pv": wl["fields"]["vorticity"]}
    kw = {"Rd": 0.3, "beta": 2.0} if wl["model"] == "quasigeostrophic" else {}
    P = _lib.lib("product")

    def run(mode):
        old = P.f2d_set_cluster(mode)
        old_sep = P.f2d_set_separable(0)
        try:
            M = engine.from_workload(wl, dt=1e-3, precision="mixed", **kw)
            lev = M.cluster_level()
            M.set_psi_from_vorticity()
            M.diagnostics()
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                M.run(3, graph=True)
            s.synchronize()
            return lev, M.var.state.cpu().numpy()
        finally:
            P.f2d_set_cluster(old)
            P.f2d_set_separable(old_sep)

    (lev_on, a), (lev_off, b) = run(levels), run(0)
    assert lev_on >= 1 and lev_off == -1
    assert P.f2d_set_cluster(-1) == 0
    assert np.array_equal(a, b)
