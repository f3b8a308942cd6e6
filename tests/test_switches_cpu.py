"""The process-wide launch switches of the C ABI (host settings, no GPU
call): defaults, query, set, the previous value returned, out-of-range
values ignored, and the exact build pinned to the reference's order of
operations (include/fluid2d_gb300.h)."""
import ctypes

import pytest

# name: (default in the product build, values to set, out-of-range values, query)
SWITCHES = {
    "f2d_set_pdl": (1, (0, 1), (), -1),
    "f2d_set_level_tiles": (0, (-1, 304, 0), (), -2),
    "f2d_set_level_threads": (0, (1, 2, 0), (3, 7), -1),
    "f2d_set_separable": (1, (0, 2, 1), (3, 9), -1),
    "f2d_set_cluster": (0, (3, 8, 0), (9, 100), -1),
    "f2d_set_l2_persist": (1, (0, 1), (2, 5), -1),
}
PINNED_IN_EXACT = {"f2d_set_separable": 0, "f2d_set_cluster": 0}


@pytest.fixture(scope="module")
def libs():
    from fluid2d_gb300 import _lib
    _lib.build()
    return {v: ctypes.CDLL(_lib.so_path(v)) for v in ("product", "exact")}


@pytest.mark.parametrize("name", sorted(SWITCHES))
def test_switch_contract(libs, name):
    default, values, bad, query = SWITCHES[name]
    f = getattr(libs["product"], name)
    f.restype, f.argtypes = ctypes.c_int, [ctypes.c_int]
    start = f(query)
    assert start == default
    prev = start
    for v in values:
        assert f(v) == prev
        now = f(query)
        assert now == (int(v != 0) if name == "f2d_set_pdl" else v)
        prev = now
    for v in bad:
        assert f(v) == prev and f(query) == prev
    f(start)
    assert f(query) == start


@pytest.mark.parametrize("name", sorted(PINNED_IN_EXACT))
def test_exact_build_keeps_the_reference_order(libs, name):
    f = getattr(libs["exact"], name)
    f.restype, f.argtypes = ctypes.c_int, [ctypes.c_int]
    want = PINNED_IN_EXACT[name]
    assert f(-1) == want
    f(1)
    assert f(-1) == want
