"""fortran_diag on GB300 (core/fortran_diag.f90)."""
from fluid2d_gb300.kernels import (computedotprod, computemax, computesum,  # noqa: F401
                                   computesumandnorm, computenormmaxu, computekemaxu,
                                   computekemaxuv, computekewithpsi)
