"""One model step inside an NVTX range, for profilers.

    python -m fluid2d_gb300.profile_step [--n 1024] [--precision fp64|mixed]
        [--coarse-level L] [--no-coarse-operator] [--steps K]
        [--ensemble N --groups G --policy P --coarse-offset D]

Builds the decaying-turbulence workload on an n x n periodic grid, sets psi,
the diagnostics and dt (CFL 0.8), runs one warm-up step, then K steps inside
the NVTX range "step" (eager launches, so a profiler sees every kernel with
its own grid) and prints the coarse level, the coarse operator's size and
the solver statistics.  With ncu: ``--nvtx --nvtx-include "step/"`` keeps
only the launches of the profiled steps.

``--ensemble N`` profiles instead the batched step of the N-instance ensemble
of ``workloads.ensemble(N, seed=4)`` (G groups of batched launches, merge
policy P; G = 0: every instance's own graph on streams; coarse switch D
levels below each instance's first allowed level), one warm-up step and K
steps inside "step".
"""
import argparse
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--precision", default="fp64", choices=("fp64", "mixed"))
    ap.add_argument("--coarse-level", type=int, default=None)
    ap.add_argument("--no-coarse-operator", action="store_true")
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--ensemble", type=int, default=0)
    ap.add_argument("--groups", type=int, default=1)
    ap.add_argument("--policy", type=int, default=1)
    ap.add_argument("--coarse-offset", type=int, default=0)
    ap.add_argument("--balanced", action="store_true")
    a = ap.parse_args(argv)
    import torch
    from fluid2d_gb300 import engine, workloads
    if a.ensemble > 0:
        E = engine.ensemble_from_workloads(workloads.ensemble(a.ensemble, seed=4),
                                           precision=a.precision, batched=a.groups > 0,
                                           groups=max(1, a.groups), policy=a.policy)
        if a.balanced and E.batch is not None:
            E.build_batch(max(1, a.groups), a.policy, balanced=True)
        if a.coarse_offset:
            E.coarse_offset(a.coarse_offset)
        E.run(1)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_push("step")
        E.run(a.steps)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        if E.batch is not None:
            print("batched launches per step %d, recorded operations %d" % E.batch_info())
        return
    M = engine.from_workload(workloads.turbulence(a.n, a.n), precision=a.precision, dt=1e-3)
    if a.coarse_level is not None:
        M.coarse_switch(a.coarse_level)
    if a.no_coarse_operator:
        M.coarse_operator(False)
    M.set_psi_from_vorticity()
    d = M.diagnostics()
    M.set_dt(0.8 * M.dx / d["maxspeed"])
    M.run(1)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("step")
    M.run(a.steps)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print("coarse level %d of %d, coarse operator %d points, solve %s"
          % (M.coarse_level, M.nlevs, M.coarse_operator(), M.solve_stats()))


if __name__ == "__main__":
    main()
