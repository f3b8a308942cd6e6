"""fluid2d_gb300.island against the reference's own Island (core/island.py,
imported over the oracle's celltocorner where the reference's sources are
present) on seeded island sets: single cells, discs, islands across the
array's edges (the neighbour count wraps), overlapping islands with
different psi0 (the later one wins), on grids with dx != dy.  No GPU."""
import contextlib
import io

import numpy as np
import pytest

from tests.conftest import reference_core


def _islands(rng, ny, nx, count):
    out = []
    for _ in range(count):
        kind = rng.integers(3)
        if kind == 0:      # one cell
            idx = (np.array([rng.integers(ny)]), np.array([rng.integers(nx)]))
        elif kind == 1:    # a disc, anywhere (also across the edges)
            yc, xc, r = rng.uniform(0, ny), rng.uniform(0, nx), rng.uniform(1.5, 6)
            y, x = np.mgrid[0:ny, 0:nx]
            idx = np.where((y + 0.5 - yc) ** 2 + (x + 0.5 - xc) ** 2 <= r * r)
        else:              # a rectangle touching the first or last row/column
            j0, i0 = rng.integers(ny - 4), rng.integers(nx - 4)
            j0 = 0 if rng.integers(2) else j0
            i1 = nx if rng.integers(2) else i0 + 4
            y, x = np.mgrid[j0:j0 + 4, i0:i1]
            idx = (y.ravel(), x.ravel())
        out.append((idx, float(rng.uniform(-2, 2))))
    return out


def _reference(core, ny, nx, dx, dy, islands):
    from oracle import refshim
    refshim.install(core)
    import island as ref_island

    class _Grid(object):
        def copy(self, obj, names):
            for k, v in zip(names, (nx, ny, dx, dy)):
                setattr(obj, k, v)

    I = ref_island.Island(None, _Grid())
    for idx, psi0 in islands:
        I.add(idx, psi0)
    with contextlib.redirect_stdout(io.StringIO()):
        I.finalize(None)
    return I.rhsp, I.psi


@pytest.mark.parametrize("seed", range(6))
def test_island_arrays_equal_the_reference(seed):
    core = reference_core("island.py")
    from fluid2d_gb300.island import Island
    rng = np.random.default_rng(seed)
    ny, nx = 38 + 2 * int(rng.integers(8)), 70
    dx, dy = 2. / (nx - 6), 1. / (ny - 6)
    isl = _islands(rng, ny, nx, 1 + seed % 4)
    want_r, want_p = _reference(core, ny, nx, dx, dy, isl)
    I = Island(nx, ny, dx, dy)
    for idx, psi0 in isl:
        I.add(idx, psi0)
    rhsp, psi = I.finalize()
    assert np.array_equal(rhsp, want_r) and np.array_equal(psi, want_p)
    assert np.count_nonzero(rhsp) > 0


def test_held_corners_and_neighbours():
    from fluid2d_gb300.island import held_corners, held_neighbours
    cells = np.zeros((6, 7), dtype=bool)
    cells[2, 3] = True
    held = held_corners(cells)
    want = np.zeros((6, 7), dtype=bool)
    want[1:3, 2:4] = True           # the four corners of cell (2, 3)
    want[-1, :] = want[:, -1] = True
    assert np.array_equal(held, want)
    k = held_neighbours(held)
    assert k[0, 0] == 2             # wraps to the held last row and column
    assert k[2, 2] == 2 and k[1, 2] == 2 and k[1, 1] == 1 and k[3, 3] == 1 and k[3, 1] == 0
