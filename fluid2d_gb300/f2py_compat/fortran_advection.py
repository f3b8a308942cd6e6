"""fortran_advection on GB300 (core/fortran_advection.f90)."""
from fluid2d_gb300.kernels import adv_upwind, adv_centered  # noqa: F401
