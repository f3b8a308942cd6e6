"""The product path has no CPU fallback and does not use the oracle (no GPU
needed; the calls are made only where no CUDA device is present):

* the drop-in kernels, their f2py-named modules and the engine's models
  raise on a machine without a GPU instead of computing on the host;
* nothing in the package, bench.py's timed paths or the smoke entry point
  imports the oracle, and no product source reads the reference's sources.
"""
import ast
import os

import numpy as np
import pytest

from tests.conftest import REFERENCE_CORE, gpu_available

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "fluid2d_gb300")

needs_no_gpu = pytest.mark.skipif(gpu_available(), reason="checks the behaviour without a GPU")


def _fields(m=16, n=20):
    msk = np.ones((m, n), dtype=np.int8)
    z = np.zeros((m, n))
    return msk, z


@needs_no_gpu
def test_drop_in_kernels_raise_without_a_gpu():
    from fluid2d_gb300 import kernels
    msk, z = _fields()
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        kernels.adv_upwind(msk, z, z.copy(), z, z, np.zeros(5), 3, 1, 5)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        kernels.fillhalo(z, 3)


@needs_no_gpu
def test_f2py_named_modules_raise_without_a_gpu():
    from fluid2d_gb300.f2py_compat import fortran_operators
    msk, z = _fields()
    with pytest.raises(RuntimeError):
        fortran_operators.celltocorner(z, z.copy())


@needs_no_gpu
def test_models_raise_without_a_gpu():
    from fluid2d_gb300 import engine
    with pytest.raises(RuntimeError):
        engine.Model("euler", nx=32, ny=32)


def _python_files(top):
    for d, _, files in os.walk(top):
        if "__pycache__" in d or "_build" in d:
            continue
        for f in files:
            if f.endswith(".py"):
                yield os.path.join(d, f)


def _imports(path):
    tree = ast.parse(open(path).read(), path)
    for node in ast.walk(tree):
        if isinstance(node, ast.Import):
            for a in node.names:
                yield a.name, node
        elif isinstance(node, ast.ImportFrom) and node.module:
            yield node.module, node


def test_package_never_imports_the_oracle():
    bad = [(p, m) for p in _python_files(PKG) for m, _ in _imports(p)
           if m == "oracle" or m.startswith("oracle.")]
    assert not bad, bad


# the functions that may load the oracle: bench.py's CPU-baseline legs and
# reference arm, and its checkers (the parity of the named workloads, started
# from the oracle's state: _oracle_start); __graft_entry__'s smoke check, and
# its build(), which compiles the oracle without running it.  The
# timed GPU runs (run_ours, _device_start, _timed_graph) are not among them.
ORACLE_USERS = {"bench.py": {"_cpu_worker", "cpu_run", "cpu_baseline", "run_reference",
                             "bench_mixed", "bench_dipole", "bench_shear", "_oracle_start"},
                "__graft_entry__.py": {"smoke", "build"}}


def test_bench_and_smoke_import_the_oracle_only_in_their_checkers():
    for name, allowed in ORACLE_USERS.items():
        path = os.path.join(ROOT, name)
        tree = ast.parse(open(path).read(), path)
        for fn in ast.walk(tree):
            if not isinstance(fn, (ast.FunctionDef, ast.AsyncFunctionDef)):
                continue
            for node in ast.walk(fn):
                mod = None
                if isinstance(node, ast.ImportFrom) and node.module:
                    mod = node.module
                elif isinstance(node, ast.Import):
                    mod = ",".join(a.name for a in node.names)
                if mod and "oracle" in mod.split("."):
                    assert fn.name in allowed, (name, fn.name)
        top = [m for m, n in _imports(path) if n in tree.body]
        assert not any(m == "oracle" or m.startswith("oracle.") for m in top), (name, top)


def test_product_sources_do_not_read_the_reference():
    paths = list(_python_files(PKG)) + [os.path.join(ROOT, f) for f in
                                        ("bench.py", "__graft_entry__.py")]
    csrc = os.path.join(PKG, "csrc")
    paths += [os.path.join(csrc, f) for f in os.listdir(csrc)]
    ref = os.path.dirname(os.path.abspath(REFERENCE_CORE))   # the reference's checkout
    bad = [p for p in paths if os.path.isfile(p) and ref in open(p).read()]
    assert not bad, bad
