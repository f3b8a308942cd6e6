"""Islands with a prescribed streamfunction (core/island.py).

An island is a set of cells (numpy index arrays, as ``np.where`` returns)
whose corner streamfunction is held at ``psi0``.  ``finalize`` gives the two
arrays the inversion uses (core/operators.py:442-444, 482-486): ``rhsp``,
subtracted from the right-hand side, and ``psi``, added to the masked
solution.  Host-side set-up; ``engine.Model.set_islands`` uploads them.
"""
import numpy as np


def _celltocorner(xr):
    """core/fortran_operators.f90:44-64 on the host: the mean of the four
    cells around each corner, rows/cols 0..m-2 (the last row and column keep
    their value)."""
    xp = np.zeros_like(xr)
    xp[:-1, :-1] = 0.25 * (((xr[:-1, :-1] + xr[:-1, 1:]) + xr[1:, :-1]) + xr[1:, 1:])
    return xp


class Island(object):
    """core/island.py:6-47 (one rank)."""

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
        for d in self.data:
            mskr = np.ones((self.nyl, self.nxl))
            mskr[d["idx"]] = 0.
            work = _celltocorner(mskr)
            mskp = np.zeros((self.nyl, self.nxl), dtype=np.int8)
            mskp[work == 1] = 1
            mskp = 1 - mskp
            vort = (np.roll(mskp, -1, axis=1) + np.roll(mskp, -1, axis=0)
                    + np.roll(mskp, +1, axis=1) + np.roll(mskp, +1, axis=0))
            z = vort * d["psi0"] / (self.dx * self.dy)
            self.rhsp[vort > 0] = z[vort > 0]
            self.psi[mskp == 1] = d["psi0"]
        return self.rhsp, self.psi

