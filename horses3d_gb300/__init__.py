"""horses3d_gb300: GB300 (sm_103a) DGSEM compressible Navier-Stokes RHS + RK3, drop-in for HORSES3D.

The compute path is the native library built by ``horses3d_gb300.build`` (CUDA kernels behind the
C ABI of include/horses3d_gb300.h). Python here is a thin host: mesh construction, the
.control-style configuration and the reference-shaped driver (``ComputeTimeDerivative``,
``TakeRK3Step``).
"""
__version__ = "0.1.0"
