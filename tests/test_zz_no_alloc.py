"""The allocation-free smoother, f2d_smoothtwicewitha_noalloc.

Some callers of this library cannot let it allocate device memory (their
memory comes from their own allocator or a fixed budget, or they may not
call cudaMalloc or synchronise the device at the point where they smooth).
f2d_smoothtwicewitha_noalloc serves them with a fixed static device work
array.  This test calls it through the C ABI and checks, on two calls in a
row, that it gives what the allocating f2d_smoothtwicewitha gives, and that
a grid too large for the fixed array is refused with F2D_ERR_LIMIT.

The file is named to be collected last, so that a run stopping at the first
failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from tests import _cases as C

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the tolerance of the product-build kernel tests


def _level_data(m, n, geom, islands, seed):
    """A multigrid level (mask, planar 5-plane A, x, b) of a realistic hierarchy."""
    from oracle import stepper
    msk0 = C.corner_mask(C.mask(m, n, geom, islands, seed))
    dx = 1. / (n - 6)
    info = stepper.gridinfo(n - 6, m - 6, dx, dx)
    levs = [stepper.Level(inf, 3, 8. / 9., 1., 'default') for inf in info]
    levs[0].set_finest(msk0)
    for k in range(1, len(levs)):
        levs[k].set_coarser(levs[k - 1])
    return levs


def _smooth(L, name, msk, A, x, b, m, n):
    import torch
    fn = getattr(L, name)
    rc = fn(ctypes.c_void_p(msk.data_ptr()), ctypes.c_void_p(A.data_ptr()),
            ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(b.data_ptr()),
            ctypes.c_double(8. / 9.), ctypes.c_int(m), ctypes.c_int(n),
            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return rc


def test_noalloc_matches_allocating_smoother_twice():
    import torch
    from fluid2d_gb300 import _lib
    L = _lib.lib("product")
    for (m, n, geom, isl, seed) in [(134, 134, "closed", 2, 1), (70, 262, "perio", 0, 2)]:
        for lev in _level_data(m, n, geom, isl, seed)[:3]:
            mv, nv = lev.mv, lev.nv
            msk = torch.from_numpy(lev.msk).cuda()
            A = torch.from_numpy(np.ascontiguousarray(
                np.moveaxis(lev.A[:, :, :5], 2, 0))).cuda()
            b = torch.from_numpy(C.field(mv, nv, seed + 5)).cuda()
            x0 = torch.from_numpy(C.field(mv, nv, seed + 6)).cuda()
            x_ref, x_new = x0.clone(), x0.clone()
            for call in range(2):  # two calls in a row on the same arrays
                assert _smooth(L, "f2d_smoothtwicewitha", msk, A, x_ref, b, mv, nv) == 0
                assert _smooth(L, "f2d_smoothtwicewitha_noalloc", msk, A, x_new, b, mv,
                               nv) == 0, L.f2d_last_error()
                torch.cuda.synchronize()
                ref, got = x_ref.cpu().numpy(), x_new.cpu().numpy()
                scale = max(1e-300, np.abs(ref).max())
                assert np.abs(got - ref).max() <= RTOL * scale, (m, n, mv, nv, call)


def test_noalloc_rejects_grids_beyond_its_fixed_array():
    import torch
    from fluid2d_gb300 import _lib
    L = _lib.lib("product")
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    msk = torch.zeros(16, dtype=torch.int8, device="cuda")
    # 2^21 points is the capacity; one row more must be refused before any launch
    rc = _smooth(L, "f2d_smoothtwicewitha_noalloc", msk, small, small, small, 2049, 1024)
    assert rc == 6  # F2D_ERR_LIMIT
    assert b"exceeds" in L.f2d_last_error()
