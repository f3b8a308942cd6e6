"""Full-size parity and error reports of the named workloads.

    python tests/validate_named.py [dipole|turbulence|shear|all] [--out FILE]

* dipole      Euler dipole, closed 128x128, 200 steps: float64 GPU path against
              the CPU oracle at every step (relative L-inf of omega and psi).
* turbulence  Euler turbulence, periodic 1024x1024: float64 GPU path against the
              CPU oracle over the first 10 steps (the parity bar: omega/psi
              within 1e-10 relative L-inf after 10 steps).
* shear       Boussinesq shear layer, 'xchannel' 2048x512, Ri = 0.1: the mixed
              form against the float64 GPU path (itself at oracle parity), per
              field relative L2 and L-inf every 100 steps over 1000 steps.

The oracle (CPU restatement of the reference) is the reference of comparison; the GPU
paths are what is measured.  A report script beside the parity tests (pytest
does not collect it).
"""
import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np


def _rel_linf(a, b):
    return float(np.abs(a - b).max() / max(1e-300, np.abs(b).max()))


def _rel_l2(a, b):
    return float(np.sqrt(((a - b) ** 2).sum()) / max(1e-300, np.sqrt((b ** 2).sum())))


def gpu_vs_oracle(wl, steps, every=1, variant="product", **kw):
    import torch
    from fluid2d_gb300 import engine
    from oracle import stepper
    p, O = stepper.from_workload(wl, **kw)
    dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
    G = engine.from_workload(wl, dt=dt, variant=variant, **kw)
    G.var.state.copy_(torch.from_numpy(O.state).cuda())
    G.diagnostics()
    names = G.var.varname_list
    rows = []
    t_cpu = t_gpu = 0.
    t = 0.
    for k in range(1, steps + 1):
        c0 = time.perf_counter()
        t = stepper.run(O, p, 1, dt, t=t)
        c1 = time.perf_counter()
        G.run(1)
        torch.cuda.synchronize()
        c2 = time.perf_counter()
        t_cpu += c1 - c0
        t_gpu += c2 - c1
        if k % every == 0 or k == steps:
            st = G.var.state.cpu().numpy()
            rows.append({"step": k, **{nm: _rel_linf(st[i], O.state[i])
                                       for i, nm in enumerate(names)
                                       if nm in ("vorticity", "psi", "u", "v", "buoyancy", "pv")}})
    return {"dt": dt, "steps": steps, "rel_linf": rows, "cpu_s": t_cpu, "gpu_s": t_gpu}


def mixed_vs_fp64(wl, steps, every, **kw):
    import torch
    from fluid2d_gb300 import engine
    A = engine.from_workload(wl, **kw)
    A.set_psi_from_vorticity()
    d = A.diagnostics()
    dt = 0.8 * min(A.dx, A.dy) / d["maxspeed"]
    A.set_dt(dt)
    B = engine.from_workload(wl, dt=dt, precision="mixed", **kw)
    B.var.state.copy_(A.var.state)
    B.diagnostics()
    names = A.var.varname_list
    rows = []
    for k in range(every, steps + 1, every):
        A.run(every)
        B.run(every)
        torch.cuda.synchronize()
        a, b = A.var.state.cpu().numpy(), B.var.state.cpu().numpy()
        row = {"step": k}
        for i, nm in enumerate(names):
            if np.abs(a[i]).max() > 0:
                row[nm] = {"rel_l2": _rel_l2(b[i], a[i]), "rel_linf": _rel_linf(b[i], a[i])}
        iu, iv = names.index("u"), names.index("v")
        nrm = np.sqrt((a[iu] ** 2).sum() + (a[iv] ** 2).sum())
        row["velocity_rel_l2"] = float(np.sqrt(((b[iu] - a[iu]) ** 2).sum()
                                               + ((b[iv] - a[iv]) ** 2).sum()) / nrm)
        rows.append(row)
    return {"dt": dt, "steps": steps, "every": every, "errors": rows}


def main(argv=None):
    from fluid2d_gb300 import workloads as W
    ap = argparse.ArgumentParser()
    ap.add_argument("which", nargs="?", default="all")
    ap.add_argument("--out", default=None)
    ap.add_argument("--turb-steps", type=int, default=10)
    ap.add_argument("--shear-steps", type=int, default=1000)
    a = ap.parse_args(argv)
    out = {}
    if a.which in ("dipole", "all"):
        out["dipole_128_200_steps_fp64_vs_oracle"] = gpu_vs_oracle(W.dipole(128, 128), 200,
                                                                   every=20)
    if a.which in ("turbulence", "all"):
        out["turbulence_1024_fp64_vs_oracle"] = gpu_vs_oracle(W.turbulence(1024, 1024), a.turb_steps,
                                                              every=1)
    if a.which in ("shear", "all"):
        out["shear_2048x512_mixed_vs_fp64"] = mixed_vs_fp64(W.shear(2048, 512), a.shear_steps,
                                                            every=100)
    txt = json.dumps(out, indent=1)
    if a.out:
        with open(a.out, "w") as f:
            f.write(txt)
    print(txt)


if __name__ == "__main__":
    sys.exit(main())
