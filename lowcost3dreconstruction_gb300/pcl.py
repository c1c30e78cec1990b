"""PCL-shaped classes over liblcr, mirroring the calls the reference tools make:

* IterativeClosestPoint      -- pcl_tools/fine_registration.cpp:105-126
* VoxelGrid                  -- pcl_tools/cloud_downsampling.cpp:73-76
* StatisticalOutlierRemoval  -- pcl_tools/outlier_removal.cpp:80-84, :92
* NormalEstimation           -- pcl_tools/normal_estimation.cpp:84-108

Same method names and argument meaning; clouds are numpy POINT_DTYPE arrays
(pcl::PointXYZRGBNormal records).  Every compute call runs on the GPU.
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from .core import Context

_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class IterativeClosestPoint:
    def __init__(self, ctx: Context | None = None, point_to_plane: bool = False):
        self._ctx = ctx or default_context()
        self._src = self._tgt = None
        self._params = Context.icp_params(point_to_plane=point_to_plane)
        self._result = None

    def setInputSource(self, cloud: np.ndarray) -> None:
        self._src = self._ctx.upload(cloud)

    def setInputTarget(self, cloud: np.ndarray) -> None:
        self._tgt = self._ctx.upload(cloud)

    def setMaxCorrespondenceDistance(self, d: float) -> None:
        self._params.max_correspondence_distance = float(d)

    def setMaximumIterations(self, n: int) -> None:
        self._params.max_iterations = int(n)

    def setTransformationEpsilon(self, eps: float) -> None:
        self._params.transformation_epsilon = float(eps)

    def setEuclideanFitnessEpsilon(self, eps: float) -> None:
        self._params.euclidean_fitness_epsilon = float(eps)

    def align(self, guess: np.ndarray | None = None) -> np.ndarray:
        """Runs the registration; returns the registered source (the `output` cloud)."""
        res, reg = self._ctx.icp(self._src, self._tgt, self._params, guess, want_registered=True)
        self._result = res
        return reg.download()

    def getFinalTransformation(self) -> np.ndarray:
        return self._result.transform

    def hasConverged(self) -> bool:
        return self._result.converged

    def getFitnessScore(self) -> float:
        return self._result.fitness


class VoxelGrid:
    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or default_context()
        self._in = None
        self._leaf = (1.0, 1.0, 1.0)

    def setInputCloud(self, cloud: np.ndarray) -> None:
        self._in = self._ctx.upload(cloud)

    def setLeafSize(self, lx: float, ly: float, lz: float) -> None:
        self._leaf = (float(lx), float(ly), float(lz))

    def filter(self) -> np.ndarray:
        return self._ctx.voxel_grid(self._in, self._leaf).download()


class StatisticalOutlierRemoval:
    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or default_context()
        self._in = None
        self._k = 1
        self._mul = 0.0
        self._negative = False

    def setInputCloud(self, cloud: np.ndarray) -> None:
        self._in = self._ctx.upload(cloud)

    def setMeanK(self, k: int) -> None:
        self._k = int(k)

    def setStddevMulThresh(self, m: float) -> None:
        self._mul = float(m)

    def setNegative(self, neg: bool) -> None:
        self._negative = bool(neg)

    def filter(self) -> np.ndarray:
        inl, outl, _ = self._ctx.sor(self._in, self._k, self._mul, want_outliers=self._negative)
        return (outl if self._negative else inl).download()


class NormalEstimation:
    def __init__(self, ctx: Context | None = None):
        self._ctx = ctx or default_context()
        self._in = None
        self._k = 0
        self._vp = (0.0, 0.0, 0.0)

    def setInputCloud(self, cloud: np.ndarray) -> None:
        self._in = self._ctx.upload(cloud)

    def setKSearch(self, k: int) -> None:
        self._k = int(k)

    def setViewPoint(self, x: float, y: float, z: float) -> None:
        self._vp = (float(x), float(y), float(z))

    def useSensorOriginAsViewPoint(self) -> None:
        # PLY clouds carry the sensor origin (0, 0, 0)
        self._vp = (0.0, 0.0, 0.0)

    def compute(self) -> np.ndarray:
        return self._ctx.normals(self._in, self._k, self._vp).download()


__all__ = ["IterativeClosestPoint", "VoxelGrid", "StatisticalOutlierRemoval", "NormalEstimation", "default_context",
           "L"]
