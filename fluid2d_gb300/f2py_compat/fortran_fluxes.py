"""fortran_fluxes on GB300 (core/fortran_fluxes.f90)."""
from fluid2d_gb300.kernels import flx_adv_upwind as adv_upwind  # noqa: F401
from fluid2d_gb300.kernels import flx_adv_centered as adv_centered  # noqa: F401
