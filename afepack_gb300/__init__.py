"""GB300-native (sm_103a) implementation of AFEPack's elliptic-solve path.

The compute lives in libafepack_gb300.so (CUDA kernels behind the C ABI of
include/afepack_gb300.h); this package holds the host-side mirror of the
reference interface (fem, amg), the mesh/DOF-numbering host code (mesh) and
the seeded workloads (workloads).
"""
from .mesh import FESpace as HostSpace, Mesh, cube_mesh, square_mesh, write_reference_mesh  # noqa: F401

__all__ = ["HostSpace", "Mesh", "cube_mesh", "square_mesh", "write_reference_mesh"]
