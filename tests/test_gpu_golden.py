"""The device engine replays the step fixtures of tests/golden/ (made by the
reference's own Python over the oracle kernels on another machine): the
initial state and dt come from the fixture, each RK3 step is compared with
the fixture's state.

Exact build: bit-identical for the closed and channel geometries (the only
reductions feeding the state are maxima); the periodic case differs by the
rounding of the psi mean and the no-slip cases by that of the mean wall
source.  Otherwise: 1e-10 of the largest value.  Covers diffusion at the
forcing stage, no-slip walls, islands with a prescribed streamfunction, line
relaxation and the advection orders.
"""
import ast
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
STEPS = sorted(p for p in glob.glob(os.path.join(HERE, "golden", "*.npz"))
               if not os.path.basename(p).startswith(("loop_", "fluxes_")))


@pytest.mark.parametrize("variant", ["exact", "product"])
@pytest.mark.parametrize("path", STEPS, ids=[os.path.basename(p)[:-4] for p in STEPS])
def test_engine_replays_reference_steps(path, variant):
    import torch
    from fluid2d_gb300 import engine
    z = np.load(path, allow_pickle=False)
    prm = ast.literal_eval(str(z["params"][0]))
    kw = {k: prm[k] for k in ("Rd", "beta", "diffusion", "Kdiff", "noslip",
                                      "hydroepsilon", "order", "flux_splitting_method") if k in prm}
    if "msknoslip" in z:
        kw["msknoslip"] = z["msknoslip"]
    G = engine.Model(prm["model"], prm["nx"], prm["ny"], prm["Lx"], prm["Ly"],
                     prm["geometry"], msk=z["msk"], gravity=prm["gravity"], dt=float(z["dt"]),
                     variant=variant, **kw)
    if "rhsp" in z:
        G.set_islands(z["rhsp"], z["psi_island"])
    states = z["states"]
    G.var.state.copy_(torch.from_numpy(states[0]).cuda())
    G.diagnostics()
    # sums that feed the state: the psi mean (periodic) and the mean wall
    # source (no-slip) are rounded in another order on the device
    exact = variant == "exact" and prm["geometry"] != "perio" and not prm.get("noslip")
    for k in range(1, len(states)):
        G.run(1)
        st = G.var.state.cpu().numpy()
        for q, nm in enumerate(G.var.varname_list):
            if exact:
                assert np.array_equal(st[q], states[k][q]), (k, nm)
            else:
                scale = max(np.abs(states[k][q]).max(), 1e-300)
                assert np.abs(st[q] - states[k][q]).max() <= 1e-10 * scale, (k, nm)
