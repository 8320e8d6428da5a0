"""fv_140823_gb300 -- GB300-native residual evaluation and Runge-Kutta stage
update for the octree finite-volume solver FV_140823.

The compute path is ``libfvgpu`` (hand-written CUDA for sm_103a behind the C
ABI in ``include/fvgpu.h``); this package holds the host-side pieces around
it: the octree mesh builder / flattener, the ctypes mirror of the reference's
RHS / RK interface, and the autograd wrapper of the adjoint.
"""
from .mesh import OctreeMesh, MeshTables, uniform_mesh, refine_by  # noqa: F401
