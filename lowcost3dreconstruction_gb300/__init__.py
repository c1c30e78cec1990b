"""GB300-native (sm_103a) implementation of the LowCost3DReconstruction
alignment path: depth back-projection, VoxelGrid, StatisticalOutlierRemoval,
NormalEstimation, IterativeClosestPoint and accumulate_clouds as hand-written
CUDA kernels behind the C ABI in include/lcr.h (liblcr.so).

Importing the package does not need a GPU; creating a Context does, and there
is no CPU fallback.
"""
from ._lib import POINT_DTYPE, LcrError  # noqa: F401

__all__ = ["POINT_DTYPE", "LcrError", "Context", "Cloud", "points_from_xyz", "xyz_of", "normals_of"]


def __getattr__(name):
    if name in ("Context", "Cloud", "points_from_xyz", "xyz_of", "normals_of", "IcpOutcome"):
        from . import core
        return getattr(core, name)
    raise AttributeError(name)
