"""CPU oracle for fluid2d_gb300 (test infrastructure only).

``oracle.oracle`` restates the reference's Fortran kernels in C (ctypes),
``oracle.stepper`` restates its Python sequencing over those kernels.
Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import it.
"""
