"""fortran_operators on GB300 (core/fortran_operators.f90)."""
from fluid2d_gb300.kernels import (computeorthogradient, celltocorner,  # noqa: F401
                                   cornertocell, add_diffusion, add_torque,
                                   computenoslipsourceterm)
