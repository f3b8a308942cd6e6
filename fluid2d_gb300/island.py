"""Islands with a prescribed streamfunction (core/island.py).

An island is a set of cells (numpy index arrays, as ``np.where`` returns)
whose corner streamfunction is held at ``psi0``.  ``finalize`` gives the two
arrays the inversion uses (core/operators.py:442-444, 482-486): ``rhsp``,
subtracted from the right-hand side, and ``psi``, added to the masked
solution.  Host-side set-up; ``engine.Model.set_islands`` uploads them.

The arrays, for each island in the order added (a later island overwrites
an earlier one where their points meet):

* the held corners are those that touch an island cell: a corner (j, i)
  joins the cells (j..j+1, i..i+1), and the last row and column, which join
  no four cells, count as held (the reference finds the corners with its
  cell-to-corner average, core/fortran_operators.f90:44-64, which leaves
  those points at zero, not at the value 1 of a corner clear of the island);
* ``psi`` is psi0 on the held corners;
* ``rhsp`` is k psi0 / (dx dy) at every point with k > 0 of its four
  neighbours held, the neighbours taken periodically over the whole array.
"""
import numpy as np


def held_corners(cells):
    """Boolean (ny, nx): the corners an island of the boolean cell array
    ``cells`` holds."""
    held = np.ones(cells.shape, dtype=bool)
    held[:-1, :-1] = cells[:-1, :-1] | cells[:-1, 1:] | cells[1:, :-1] | cells[1:, 1:]
    return held


def held_neighbours(held):
    """int8 (ny, nx): how many of each point's four neighbours are held
    (periodic wrap in both directions)."""
    h = np.pad(held.astype(np.int8), 1, mode="wrap")
    return h[:-2, 1:-1] + h[2:, 1:-1] + h[1:-1, :-2] + h[1:-1, 2:]


class Island(object):
    """core/island.py:6-47 (one rank): ``add`` islands, then ``finalize``."""

    def __init__(self, nxl, nyl, dx, dy):
        self.nxl, self.nyl, self.dx, self.dy = nxl, nyl, dx, dy
        self.rhsp = np.zeros((nyl, nxl))
        self.psi = np.zeros((nyl, nxl))
        self.data = []

    @classmethod
    def for_model(cls, model):
        return cls(model.nxl, model.nyl, model.dx, model.dy)

    def add(self, idx, psi0):
        self.data.append({"idx": idx, "psi0": psi0})

    @property
    def nbisland(self):
        return len(self.data)

    def finalize(self, mskp_model=None):
        """(rhsp, psi); ``mskp_model`` is accepted for the reference's
        signature and not used (nor is it there)."""
        area = self.dx * self.dy
        for isl in self.data:
            cells = np.zeros((self.nyl, self.nxl), dtype=bool)
            cells[isl["idx"]] = True
            held = held_corners(cells)
            k = held_neighbours(held)
            src = k > 0
            self.rhsp[src] = k[src] * isl["psi0"] / area
            self.psi[held] = isl["psi0"]
        return self.rhsp, self.psi
