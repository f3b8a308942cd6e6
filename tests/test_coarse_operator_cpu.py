"""The coarse part of a multigrid cycle started from x = 0 is a fixed linear
map of the coarse level's interior right-hand side: the design of the product
build's coarse operator, checked here on the oracle's own cycle (no GPU).  The
map is built as the GPU builds it, column by column from unit vectors with
their periodic images (the halo the restriction leaves in b); applied to
random right-hand sides it reproduces the V- and F-cycles to rounding, halo
included (every halo point of x is the image of an interior point)."""
import numpy as np
import pytest

from tests import _cases as C

NH = 3


def _images(interior):
    return np.pad(interior, NH, mode="wrap")


def _cycle(G, lev, mode, b):
    G.x[lev][:, :] = 0.
    G.b[lev][:, :] = b
    if mode == "V":
        G.Vcycle(lev)
    else:
        G.Fcycle(lev)
    return G.x[lev].copy()


@pytest.mark.parametrize("geom,isl,seed", [("perio", 0, 3), ("closed", 1, 5), ("xchannel", 0, 7)])
@pytest.mark.parametrize("mode", ["V", "F"])
def test_coarse_cycle_is_its_linear_map(geom, isl, seed, mode):
    from oracle import stepper
    m = n = 70
    msk = C.corner_mask(C.mask(m, n, geom, isl, seed))
    pp = {'nh': NH, 'n': n - 6, 'm': m - 6, 'omega': 8. / 9., 'dx': 1. / 64, 'dy': 1. / 64}
    G = stepper.Gmg(pp, msk * 1.)
    lev = G.nlevs - 2                      # 8 x 8 interior points above the 4 x 4 deepest
    g = G.grid[lev]
    m2, n2 = g.mv - 2 * NH, g.nv - 2 * NH
    npts = m2 * n2
    op = np.zeros((npts, npts))
    for k in range(npts):
        e = np.zeros((m2, n2))
        e[k // n2, k % n2] = 1.
        op[:, k] = _cycle(G, lev, mode, _images(e))[NH:-NH, NH:-NH].ravel()
    rng = np.random.default_rng(seed)
    for _ in range(3):
        bi = rng.standard_normal((m2, n2))
        want = _cycle(G, lev, mode, _images(bi))
        got = _images((op @ bi.ravel()).reshape(m2, n2))
        scale = np.abs(want).max()
        assert scale > 0
        assert np.abs(got - want).max() <= 1e-12 * scale
