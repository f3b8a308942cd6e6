"""The oracle's timing build (the CPU baseline bench.py times: -O3 with
multiply-adds contracted into FMA) computes the same steps as its parity
build (no contraction, the Fortran's rounding) to rounding: the timed CPU
path does the reference's work, not less.  Each build runs in its own
process (the build is chosen when the library is first loaded)."""
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import json, sys
import numpy as np
sys.path.insert(0, %r)
from fluid2d_gb300 import workloads as W
from oracle import oracle, stepper
assert oracle.variant() == sys.argv[1]
wl = W.turbulence(64, 64, seed=2)
p, O = stepper.from_workload(wl)
dt = 0.8 * min(O.grid.dx, O.grid.dy) / O.diags["maxspeed"]
stepper.run(O, p, 3, dt)
np.save(sys.argv[2], O.state)
"""


def _run(variant, out):
    env = dict(os.environ, F2D_ORACLE_VARIANT=variant)
    r = subprocess.run([sys.executable, "-c", SCRIPT % ROOT, variant, out], env=env,
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


def test_timing_build_steps_like_the_parity_build(tmp_path):
    from oracle import oracle
    oracle.build()
    a = _run("parity", str(tmp_path / "parity.npy"))
    b = _run("timing", str(tmp_path / "timing.npy"))
    assert a.shape == b.shape
    for k in range(4):          # vorticity, psi, u, v
        scale = np.abs(a[k]).max()
        assert scale > 0
        assert np.abs(a[k] - b[k]).max() <= 1e-10 * scale, k
