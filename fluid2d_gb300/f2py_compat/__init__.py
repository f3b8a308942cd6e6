"""Drop-in replacements for Fluid2d's f2py extension modules.

Put this directory on ``sys.path`` ahead of the reference's ``core/`` and
``core/gmg/`` (``fluid2d_gb300.f2py_compat.install()`` does it) and the
reference's ``operators.py``, ``fluxes.py``, ``gmg/*.py`` and models import
the GB300 kernels under the module names they already use:
``fortran_advection``, ``fortran_operators``, ``fortran_diag``,
``fortran_fluxes`` and ``gmg.fortran_multigrid``.

Every routine the reference's Python calls is provided.  Not provided: the
routines it never calls (``smoothoncewitha`` and ``celltocornerbicubic``
and ``computewallshear`` appear only in commented-out lines,
core/gmg/level.py:354-355, core/operators.py:441, core/operators.py:241;
``computenoslipsourceterm_regularized`` nowhere), and the MPI halo packers
``halotobuffer``, ``buffertohalo`` and ``buffertodomain``
(core/gmg/fortran_multigrid.f90:549-703), which serve the domain
decomposition this single-GPU path does not do.
"""
import os
import sys

PATH = os.path.dirname(os.path.abspath(__file__))


def install():
    """Prepend the replacement modules to sys.path (idempotent)."""
    if PATH not in sys.path:
        sys.path.insert(0, PATH)
    repo = os.path.dirname(os.path.dirname(PATH))
    if repo not in sys.path:
        sys.path.insert(0, repo)
    return PATH
