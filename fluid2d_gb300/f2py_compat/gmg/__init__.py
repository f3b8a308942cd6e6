"""``gmg`` package seen by Fluid2d when the GB300 kernels are installed.

Its ``fortran_multigrid`` module is the GB300 one (this directory); every
other submodule (``gmg.level``, ``gmg.hierarchy``, ``gmg.halo``, ...) is
found in the reference's own ``core/gmg`` directory on ``sys.path``, which
is appended to this package's search path.  Like core/gmg/__init__.py, the
package re-exports the kernels.
"""
import os
import sys

_here = os.path.dirname(os.path.abspath(__file__))
for _entry in list(sys.path):
    _cand = os.path.join(os.path.abspath(_entry or "."), "gmg")
    if _cand != _here and os.path.exists(os.path.join(_cand, "level.py")):
        __path__.append(_cand)

from .fortran_multigrid import *  # noqa: E402,F401,F403
