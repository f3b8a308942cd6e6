"""The premise of the product build's column-form sweeps on stored levels
(`k_sweepu`, `k_stencil_samples`, `k_uniform_flags`), checked on the oracle's
own hierarchy (no GPU): the Galerkin coarsening (core/gmg/fortran_multigrid.f90:
706-811, core/gmg/level.py:304-330) does the same arithmetic at every point of a
fluid region, so the coarse operators' stencils agree bit for bit away from
walls and, where the spacing keeps the arithmetic symmetric, have the uniform
form the device flags look for (four equal corners, equal vertical and equal
horizontal edges).  The device takes the stencil that at least 8 of 16 sampled
points share and flags each point whose stored planes equal it exactly, so a
hierarchy where the premise fails only loses speed: no point is flagged and the
general expression runs everywhere (the last case here)."""
import numpy as np
import pytest

from tests import _cases as C

NH = 3


def _levels(m, n, geom, dx, isl=0, seed=3):
    from oracle import stepper
    msk = C.corner_mask(C.mask(m + 2 * NH, n + 2 * NH, geom, isl, seed))
    pp = {'nh': NH, 'n': n, 'm': m, 'omega': 8. / 9., 'dx': dx, 'dy': dx}
    G = stepper.Gmg(pp, msk * 1.)
    return G.grid[1:]


def _uniform_stencils(g):
    """(fluid points of rows/cols 1..m-2, {stencil: count} over those with the
    uniform form); a stencil is (corner, vertical edge, horizontal edge,
    centre), planes SW, S, SE, W, C as the hierarchy keeps them."""
    A = g.A
    J, I = np.nonzero(g.msk[1:-1, 1:-1])
    J, I = J + 1, I + 1
    c = A[J, I, 0]
    ok = ((A[J, I, 2] == c) & (A[J + 1, I - 1, 2] == c) & (A[J + 1, I + 1, 0] == c)
          & (A[J, I, 1] == A[J + 1, I, 1]) & (A[J, I, 3] == A[J, I + 1, 3]))
    keys = np.stack([c, A[J, I, 1], A[J, I, 3], A[J, I, 4]], 1)[ok]
    if not len(keys):
        return len(J), {}
    u, cnt = np.unique(keys, axis=0, return_counts=True)
    return len(J), {tuple(k): int(n) for k, n in zip(u, cnt)}


@pytest.mark.parametrize("dx", [1. / 64, 1. / 100, 1. / 3, 2 * np.pi / 128])
def test_periodic_levels_have_one_uniform_stencil(dx):
    for g in _levels(64, 64, "perio", dx):
        npts, st = _uniform_stencils(g)
        assert len(st) == 1, (g.lev, len(st))
        assert list(st.values())[0] == npts


@pytest.mark.parametrize("geom,isl", [("closed", 0), ("xchannel", 0), ("closed", 1)])
def test_walled_levels_share_the_interior_stencil(geom, isl):
    for g in _levels(128, 128, geom, 1. / 128, isl=isl):
        npts, st = _uniform_stencils(g)
        assert len(st) == 1, (g.lev, len(st))
        if g.m >= 16:  # the wall rows are a small part of the level
            assert list(st.values())[0] >= npts // 2, (g.lev, st, npts)


def test_asymmetric_rounding_leaves_no_point_flagged():
    lv = _levels(128, 128, "perio", 0.3)
    assert _uniform_stencils(lv[0])[1]         # level 1 is exact
    for g in lv[1:]:
        assert _uniform_stencils(g)[1] == {}, g.lev
