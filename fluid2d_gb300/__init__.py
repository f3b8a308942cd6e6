"""fluid2d_gb300 -- GB300-native (sm_103a) time-step hot path of Fluid2d.

* ``fluid2d_gb300.kernels``      the reference's f2py kernel modules on the GPU
* ``fluid2d_gb300.f2py_compat``  drop-in module names for the reference's Python
* ``fluid2d_gb300.engine``       device-resident multigrid and model steppers
"""
__version__ = "1.0"
