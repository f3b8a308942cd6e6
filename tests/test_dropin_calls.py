"""CPU checks of the drop-in boundary (no GPU call is made):

* the modules of fluid2d_gb300/f2py_compat are found under the bare names
  the reference imports (install.sh:44-46) and export every routine its
  Python calls (tests/golden/dropin_calls.json);
* where the reference's sources are present, its Python over the oracle
  replays fixtures with exactly the kernel calls recorded there, which are
  the oracle stepper's (tests/golden/make_dropin_calls.py).
"""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
from tests.conftest import REFERENCE_CORE  # noqa: E402


def calls():
    with open(os.path.join(GOLDEN, "dropin_calls.json")) as f:
        return json.load(f)


def test_every_step_fixture_and_scheme_is_recorded():
    rec = calls()
    names = [f[:-4] for f in os.listdir(GOLDEN)
             if f.endswith(".npz") and not f.startswith(("loop_", "fluxes_"))]
    assert names and all(n in rec for n in names)
    for s in ("EF", "LF", "Heun", "AB2", "AB3", "LFAM3", "RK3", "RK4_LS"):
        assert "euler_closed_32:%s" % s in rec
    assert all(r["calls"] > 1000 and len(r["sha256"]) == 64 for r in rec.values())


def test_modules_resolve_by_bare_name():
    routines = sorted({f.split("(")[0] for r in calls().values() for f in r["forms"]})
    code = """
import importlib, json, os, sys
sys.path.insert(0, %r)
from fluid2d_gb300 import f2py_compat
path = f2py_compat.install()
out = {}
for q in json.loads(%r):
    mod, fn = q.rsplit(".", 1)
    m = importlib.import_module(mod)
    out[q] = [os.path.dirname(os.path.abspath(m.__file__)).startswith(path), hasattr(m, fn)]
print(json.dumps(out))
""" % (ROOT, json.dumps(routines))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert set(res) == set(routines)
    bad = [q for q, (inside, present) in res.items() if not (inside and present)]
    assert not bad, bad


@pytest.mark.skipif(not os.path.isdir(REFERENCE_CORE), reason="reference sources absent")
@pytest.mark.parametrize("name,scheme", [("boussinesq_xchannel_64x16_noslip", None),
                                         ("qg_xchannel_64x32_islands", None),
                                         ("euler_closed_32", "AB3")])
def test_reference_calls_match_record(name, scheme):
    sys.path.insert(0, GOLDEN)
    import make_dropin_calls as D
    path = os.path.join(GOLDEN, name + ".npz")
    key = name if scheme is None else "%s:%s" % (name, scheme)
    got = D.record(REFERENCE_CORE, path, scheme, D.SCHEME_STEPS if scheme else None)
    ref = calls()[key]
    assert got["sha256"] == ref["sha256"] and got["calls"] == ref["calls"]
