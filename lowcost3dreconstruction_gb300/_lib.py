"""ctypes binding of liblcr (include/lcr.h).

The shared library is the product; this module only declares its C
signatures and turns status codes into exceptions.  There is no fallback: if
liblcr.so is missing the import of the compute API raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "liblcr.so"

# Byte-compatible with pcl::PointXYZRGBNormal and lcr_point (48 bytes).
POINT_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("pad0", "<f4"),
    ("normal_x", "<f4"), ("normal_y", "<f4"), ("normal_z", "<f4"), ("pad1", "<f4"),
    ("b", "u1"), ("g", "u1"), ("r", "u1"), ("a", "u1"),
    ("curvature", "<f4"), ("pad2", "<f4", (2,)),
])
assert POINT_DTYPE.itemsize == 48

STATUS = {
    0: "LCR_OK", 1: "LCR_ERR_INVALID_ARG", 2: "LCR_ERR_EMPTY", 3: "LCR_ERR_NO_CORRESPONDENCES",
    4: "LCR_NOT_CONVERGED", 5: "LCR_ERR_CUDA", 6: "LCR_ERR_TIMEOUT", 7: "LCR_ERR_OOM", 8: "LCR_ERR_IO",
    9: "LCR_ERR_TOO_FEW_POINTS", 10: "LCR_ERR_NO_DEVICE",
}
OK, INVALID_ARG, EMPTY, NO_CORRESPONDENCES, NOT_CONVERGED = 0, 1, 2, 3, 4
CUDA_ERR, TIMEOUT, OOM, IO, TOO_FEW_POINTS, NO_DEVICE = 5, 6, 7, 8, 9, 10

KINECT_V1, KINECT_V2, PINHOLE_F32 = 0, 1, 2
ICP_POINT_TO_POINT, ICP_POINT_TO_PLANE = 0, 1
(ICP_STATE_NOT_CONVERGED, ICP_STATE_ITERATIONS, ICP_STATE_TRANSFORM, ICP_STATE_ABS_MSE, ICP_STATE_REL_MSE,
 ICP_STATE_NO_CORRESPONDENCES, ICP_STATE_STOPPED) = range(7)
NORMALS_FLIP_ALL, NORMALS_KEEP_NEIGHBOURS = 1, 2
ACCUM_ALL = 1


class LcrError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class DepthParams(C.Structure):
    _fields_ = [("model", C.c_int), ("width", C.c_int), ("height", C.c_int), ("frames", C.c_int),
                ("fx", C.c_double), ("fy", C.c_double), ("cx", C.c_double), ("cy", C.c_double),
                ("depth_min", C.c_double), ("depth_max", C.c_double),
                ("roi_left", C.c_int), ("roi_right", C.c_int), ("roi_top", C.c_int), ("roi_bottom", C.c_int),
                ("scale", C.c_double), ("normals", C.c_int),
                ("r", C.c_uint8), ("g", C.c_uint8), ("b", C.c_uint8), ("pad", C.c_uint8)]


class SorStats(C.Structure):
    _fields_ = [("mean", C.c_double), ("stddev", C.c_double), ("threshold", C.c_double),
                ("valid", C.c_size_t), ("kept", C.c_size_t), ("removed", C.c_size_t)]


KT_SOR_KNN, KT_NORMALS_KNN, KT_ENCODE, KT_ICP_SEARCH = 0, 1, 2, 3
POSENET_PARAMS, POSENET_POINTS = 1323401, 1024


class IcpParams(C.Structure):
    _fields_ = [("max_correspondence_distance", C.c_double), ("max_iterations", C.c_int),
                ("transformation_epsilon", C.c_double), ("euclidean_fitness_epsilon", C.c_double),
                ("method", C.c_int), ("compute_fitness", C.c_int), ("stop_iteration", C.c_int),
                ("stop_rms", C.c_double)]


class IcpResult(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("transform64", C.c_double * 16), ("converged", C.c_int),
                ("iterations", C.c_int), ("state", C.c_int), ("n_correspondences", C.c_int),
                ("fitness", C.c_double), ("mse", C.c_double)]


class AdamwParams(C.Structure):
    _fields_ = [("lr", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("eps", C.c_float),
                ("weight_decay", C.c_float)]


class SynthParams(C.Structure):
    _fields_ = [("yaw_deg", C.c_float), ("tilt_deg", C.c_float), ("translation", C.c_float), ("noise", C.c_int)]


class RenderParams(C.Structure):
    _fields_ = [("model", C.c_int), ("width", C.c_int), ("height", C.c_int), ("fx", C.c_double), ("fy", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("samples_per_pixel", C.c_float)]


class Tune(C.Structure):
    _fields_ = [("sor_warps", C.c_int), ("normals_warps", C.c_int), ("icp_blocks_per_sm", C.c_int)]


class TuneReport(C.Structure):
    _fields_ = [("chosen", Tune), ("from_cache", C.c_int), ("sor_ms", C.c_double * 8),
                ("normals_ms", C.c_double * 8), ("icp_ms", C.c_double * 8)]


class SrParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("frames", C.c_int), ("factor", C.c_int),
                ("ecc_iterations", C.c_int), ("ecc_epsilon", C.c_double)]


_VP = C.c_void_p
_SIGS = {
    "lcr_ctx_create": (C.c_int, [C.POINTER(_VP), C.c_int]),
    "lcr_ctx_destroy": (None, [_VP]),
    "lcr_last_error": (C.c_char_p, [_VP]),
    "lcr_status_string": (C.c_char_p, [C.c_int]),
    "lcr_ctx_synchronize": (C.c_int, [_VP]),
    "lcr_ctx_stream": (_VP, [_VP]),
    "lcr_ctx_launch_count": (C.c_uint64, [_VP]),
    "lcr_kernel_timing": (C.c_int, [_VP, C.c_int]),
    "lcr_kernel_time": (C.c_int, [_VP, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "lcr_cloud_upload": (C.c_int, [_VP, _VP, C.c_size_t, C.POINTER(_VP)]),
    "lcr_cloud_upload_xyz": (C.c_int, [_VP, _VP, C.c_size_t, C.POINTER(_VP)]),
    "lcr_cloud_from_device": (C.c_int, [_VP, _VP, C.c_size_t, C.POINTER(_VP)]),
    "lcr_cloud_size": (C.c_size_t, [_VP]),
    "lcr_cloud_download": (C.c_int, [_VP, _VP, _VP, C.c_size_t]),
    "lcr_cloud_neighbours": (C.c_int, [_VP, _VP, C.POINTER(C.c_int), _VP]),
    "lcr_cloud_free": (None, [_VP, _VP]),
    "lcr_cloud_concat": (C.c_int, [_VP, _VP, _VP, C.POINTER(_VP)]),
    "lcr_backproject": (C.c_int, [_VP, _VP, C.POINTER(DepthParams), C.POINTER(_VP)]),
    "lcr_backproject_device": (C.c_int, [_VP, _VP, C.POINTER(DepthParams), C.POINTER(_VP)]),
    "lcr_burst_fuse": (C.c_int, [_VP, _VP, C.POINTER(DepthParams), _VP]),
    "lcr_backproject_into": (C.c_int, [_VP, _VP, C.POINTER(DepthParams), _VP, C.c_size_t, _VP]),
    "lcr_voxel_grid": (C.c_int, [_VP, _VP, C.c_float, C.c_float, C.c_float, C.POINTER(_VP)]),
    "lcr_sor": (C.c_int, [_VP, _VP, C.c_int, C.c_double, C.POINTER(_VP), C.POINTER(_VP), C.POINTER(SorStats)]),
    "lcr_sor_distances": (C.c_int, [_VP, _VP, C.c_int, _VP, C.POINTER(SorStats)]),
    "lcr_normals": (C.c_int, [_VP, _VP, C.c_int, _VP, C.c_int, C.POINTER(_VP)]),
    "lcr_icp_params_default": (None, [C.POINTER(IcpParams)]),
    "lcr_icp": (C.c_int, [_VP, _VP, _VP, C.POINTER(IcpParams), _VP, C.POINTER(IcpResult), C.POINTER(_VP)]),
    "lcr_icp_batch": (C.c_int, [_VP, _VP, _VP, C.c_size_t, C.POINTER(IcpParams), _VP, _VP]),
    "lcr_correspondences": (C.c_int, [_VP, _VP, _VP, _VP, C.c_double, _VP, _VP]),
    "lcr_knn": (C.c_int, [_VP, _VP, _VP, C.c_int, C.c_float, _VP, _VP]),
    "lcr_accumulate": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_int, C.c_double, C.c_int, C.POINTER(_VP),
                                 C.POINTER(_VP)]),
    "lcr_crop_redundant": (C.c_int, [_VP, _VP, _VP, C.c_double, _VP]),
    "lcr_remove_nan": (C.c_int, [_VP, _VP, C.POINTER(_VP)]),
    "lcr_transform": (C.c_int, [_VP, _VP, _VP, C.POINTER(_VP)]),
    "lcr_centroid": (C.c_int, [_VP, _VP, _VP]),
    "lcr_centroid_align": (C.c_int, [_VP, _VP, _VP, C.c_double, C.c_double, C.c_double, C.c_double,
                                     C.POINTER(_VP), _VP]),
    "lcr_crop_box": (C.c_int, [_VP, _VP, _VP, _VP, C.POINTER(_VP), C.POINTER(_VP)]),
    "lcr_euclidean_clusters": (C.c_int, [_VP, _VP, C.c_double, C.c_size_t, C.c_size_t, _VP, C.POINTER(C.c_size_t),
                                         C.POINTER(_VP), C.POINTER(_VP)]),
    "lcr_plane_segment": (C.c_int, [_VP, _VP, C.c_double, C.c_int, C.c_uint64, _VP, C.POINTER(C.c_size_t),
                                    C.POINTER(_VP), C.POINTER(_VP)]),
    "lcr_super_resolve": (C.c_int, [_VP, _VP, C.POINTER(SrParams), _VP, _VP, _VP, _VP]),
    "lcr_super_resolve_f32": (C.c_int, [_VP, _VP, C.POINTER(SrParams), _VP, _VP, _VP, _VP]),
    "lcr_tune_get": (C.c_int, [_VP, C.POINTER(Tune)]),
    "lcr_tune_set": (C.c_int, [_VP, C.POINTER(Tune)]),
    "lcr_autotune": (C.c_int, [_VP, _VP, _VP, C.c_char_p, C.POINTER(TuneReport)]),
    "lcr_synthetic_pairs": (C.c_int, [_VP, C.c_uint64, C.c_size_t, C.c_int, C.POINTER(SynthParams), _VP, _VP,
                                      _VP]),
    "lcr_synthetic_depth": (C.c_int, [_VP, C.c_uint64, C.c_size_t, C.POINTER(SynthParams), C.POINTER(RenderParams),
                                      _VP, _VP, _VP, _VP]),
    "lcr_synthetic_turntable": (C.c_int, [_VP, C.c_uint64, C.c_int, C.c_float, C.POINTER(RenderParams), C.c_float,
                                          C.c_int, _VP, _VP]),
    "lcr_rmse_batch": (C.c_int, [_VP, _VP, C.c_size_t, _VP, _VP, _VP]),
    "lcr_posenet_create": (C.c_int, [_VP, C.c_uint64, C.POINTER(_VP)]),
    "lcr_posenet_free": (C.c_int, [_VP, _VP]),
    "lcr_posenet_get_params": (C.c_int, [_VP, _VP, _VP]),
    "lcr_posenet_set_params": (C.c_int, [_VP, _VP, _VP]),
    "lcr_posenet_sample": (C.c_int, [_VP, _VP, C.c_size_t, C.c_uint64, _VP, _VP]),
    "lcr_posenet_forward": (C.c_int, [_VP, _VP, _VP, C.c_size_t, C.c_int, _VP, _VP, _VP]),
    "lcr_posenet_gradients": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, _VP, _VP]),
    "lcr_posenet_train_step": (C.c_int, [_VP, _VP, _VP, _VP, _VP, C.c_size_t, C.c_uint64, C.POINTER(AdamwParams),
                                         _VP]),
    "lcr_posenet_propose": (C.c_int, [_VP, _VP, _VP, _VP, C.c_size_t, C.c_uint64, _VP]),
    "lcr_ply_read": (C.c_int, [C.c_char_p, C.POINTER(_VP), C.POINTER(C.c_size_t)]),
    "lcr_ply_write": (C.c_int, [C.c_char_p, _VP, C.c_size_t, C.c_int]),
    "lcr_ply_last_error": (C.c_char_p, []),
    "lcr_free": (None, [_VP]),
}

_lib = None


def exported_symbols() -> list[str]:
    return list(_SIGS)


def load(path: os.PathLike | str | None = None) -> C.CDLL:
    """Load liblcr.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with lowcost3dreconstruction_gb300.build "
                          "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def read_ply(path: os.PathLike | str) -> np.ndarray:
    """pcl::io::loadPLYFile equivalent (host only; no GPU needed)."""
    lib = load()
    p = C.c_void_p()
    n = C.c_size_t()
    st = lib.lcr_ply_read(str(path).encode(), C.byref(p), C.byref(n))
    if st != OK:
        raise LcrError(st, lib.lcr_ply_last_error().decode())
    try:
        buf = (C.c_char * (n.value * POINT_DTYPE.itemsize)).from_address(p.value)
        return np.frombuffer(bytes(buf), dtype=POINT_DTYPE).copy()
    finally:
        lib.lcr_free(p)


def write_ply(path: os.PathLike | str, pts: np.ndarray, binary: bool = True) -> None:
    """pcl::io::savePLYFileBinary equivalent (binary_little_endian), or ascii."""
    lib = load()
    pts = np.ascontiguousarray(pts, dtype=POINT_DTYPE)
    st = lib.lcr_ply_write(str(path).encode(), ptr(pts), len(pts), 1 if binary else 0)
    if st != OK:
        raise LcrError(st, lib.lcr_ply_last_error().decode())
