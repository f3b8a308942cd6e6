"""gmg.fortran_multigrid on GB300 (core/gmg/fortran_multigrid.f90)."""
from fluid2d_gb300.kernels import (smoothtwicewitha, smoothtridiag,  # noqa: F401
                                   computeresidualwitha, fillhalo, interpolate, restrict,
                                   coarsenmatrix, computenorm, computeinner)
