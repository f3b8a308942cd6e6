"""The device flux diagnostic (core/fluxes.py:100-213) against the fixtures
made by the reference's own Fluxes class over the oracle kernels.

Each fixture holds the initial state, the time step and the rev/irr flux
planes after each of two model steps.  The exact build reproduces them bit
for bit (every kernel on the path is the drop-in kernel of its Fortran
routine, and the RK combinations use numpy's evaluation order); the product
build agrees to 1e-9 of the largest flux.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
NAMES = ["fluxes_euler_closed_32", "fluxes_boussinesq_xchannel_64x16"]


def _workload(z):
    from fluid2d_gb300 import workloads as W
    model = str(z["model"][0])
    m, n = z["msk"].shape
    if model == "euler":
        return W.dipole(n - 6, m - 6, seed=1)
    return W.shear(n - 6, m - 6, seed=3, delta=0.1)


@pytest.mark.parametrize("variant", ["exact", "product"])
@pytest.mark.parametrize("name", NAMES)
def test_diag_fluxes_matches_reference(name, variant):
    import torch
    from fluid2d_gb300 import engine
    z = np.load(os.path.join(HERE, "golden", name + ".npz"), allow_pickle=False)
    wl = _workload(z)
    assert np.array_equal(wl["msk"], z["msk"])
    G = engine.from_workload(wl, variant=variant, dt=float(z["dt"]))
    G.var.state.copy_(torch.from_numpy(z["init_state"]).cuda())
    G.diagnostics()
    G.flux_setup()
    assert G.fullflx_list == [str(s) for s in z["names"]]
    for k in range(z["flx"].shape[0]):
        G.run(1)
        flx = G.diag_fluxes().cpu().numpy()
        ref = z["flx"][k]
        if variant == "exact":
            bad = [G.fullflx_list[q] for q in range(ref.shape[0])
                   if not np.array_equal(flx[q], ref[q])]
            assert not bad, (k, bad)
        else:
            for q in range(ref.shape[0]):
                scale = max(np.abs(ref[q]).max(), 1e-300)
                assert np.abs(flx[q] - ref[q]).max() <= 1e-9 * scale, (k, G.fullflx_list[q])
    st = G.var.state.cpu().numpy()
    if variant == "exact":
        assert np.array_equal(st, z["final_state"])
    else:
        assert np.abs(st - z["final_state"]).max() <= 1e-10 * np.abs(z["final_state"]).max()


def test_qg_has_no_flux_diagnostic():
    from fluid2d_gb300 import engine, _lib
    from fluid2d_gb300 import workloads as W
    wl = W.dipole(32, 32)
    wl["model"] = "quasigeostrophic"
    wl["fields"] = {"pv": wl["fields"]["vorticity"]}
    G = engine.from_workload(wl, Rd=0.3)
    with pytest.raises(_lib.F2DError):
        G.flux_setup()
