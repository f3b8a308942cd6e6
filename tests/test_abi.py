"""The C ABI library builds for sm_103a, loads, and exports every symbol
that include/fluid2d_gb300.h declares (no GPU needed: nothing is called)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = []
    inc = os.path.join(ROOT, "include")
    for f in sorted(os.listdir(inc)):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            syms += re.findall(r"\b(f2d_\w+)\s*\(", txt)
    return sorted(set(syms))


@pytest.fixture(scope="module")
def libs():
    from fluid2d_gb300 import _lib
    _lib.build()
    return [ctypes.CDLL(_lib.so_path(v)) for v in ("product", "exact")]


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "f2d_adv_upwind" in syms and "f2d_smoothtwicewitha" in syms
    assert len(syms) >= 25


def test_library_exports_every_declared_symbol(libs):
    for L in libs:
        missing = [s for s in declared_symbols() if not hasattr(L, s)]
        assert not missing, missing


def test_exact_flag(libs):
    prod, exact = libs
    prod.f2d_exact_arithmetic.restype = ctypes.c_int
    exact.f2d_exact_arithmetic.restype = ctypes.c_int
    assert prod.f2d_exact_arithmetic() == 0
    assert exact.f2d_exact_arithmetic() == 1


def test_python_signatures_cover_header():
    from fluid2d_gb300 import _lib
    known = set(_lib.SIGNATURES) | set(_lib.EXTRA)
    try:
        from fluid2d_gb300 import _abi_ext
        known |= set(_abi_ext.SIGNATURES)
    except ImportError:
        pass
    missing = [s for s in declared_symbols() if s not in known]
    assert not missing, missing
