"""ctypes wrapper of liboracle.so -- TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
parity reference and CPU timing baseline; never by the library.  Parity is UNPINNED (the
reference has no tests or golden vectors and its PCL/OpenCV code cannot be
built here); see oracle.h for what each function restates.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

POINT_DTYPE = np.dtype([
    ("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("pad0", "<f4"),
    ("normal_x", "<f4"), ("normal_y", "<f4"), ("normal_z", "<f4"), ("pad1", "<f4"),
    ("b", "u1"), ("g", "u1"), ("r", "u1"), ("a", "u1"),
    ("curvature", "<f4"), ("pad2", "<f4", (2,)),
])


class BpParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("fx", C.c_double), ("fy", C.c_double),
                ("cx", C.c_double), ("cy", C.c_double), ("depth_min", C.c_double), ("depth_max", C.c_double),
                ("roi_left", C.c_int), ("roi_right", C.c_int), ("roi_top", C.c_int), ("roi_bottom", C.c_int),
                ("scale", C.c_double), ("normals", C.c_int), ("r", C.c_uint8), ("g", C.c_uint8),
                ("b", C.c_uint8), ("pad", C.c_uint8)]


class IcpParams(C.Structure):
    _fields_ = [("max_corr_dist", C.c_double), ("max_iterations", C.c_int), ("transformation_epsilon", C.c_double),
                ("euclidean_fitness_epsilon", C.c_double), ("point_to_plane", C.c_int),
                ("min_correspondences", C.c_int)]


class IcpResult(C.Structure):
    _fields_ = [("transform", C.c_double * 16), ("converged", C.c_int), ("iterations", C.c_int),
                ("state", C.c_int), ("n_corr_last", C.c_int), ("fitness", C.c_double), ("mse_last", C.c_double)]


_VP = C.c_void_p
_SIGS = {
    "orc_version": (C.c_int, []),
    "orc_set_threads": (None, [C.c_int]),
    "orc_ze_mean_u16": (None, [_VP, C.c_int, C.c_size_t, _VP]),
    "orc_ze_mean_f32": (None, [_VP, C.c_int, C.c_size_t, _VP]),
    "orc_image_normals_u16": (None, [_VP, C.c_int, C.c_int, _VP]),
    "orc_backproject_v1": (C.c_size_t, [_VP, C.POINTER(BpParams), C.c_int, _VP]),
    "orc_backproject_v2": (C.c_size_t, [_VP, C.POINTER(BpParams), _VP]),
    "orc_knn": (C.c_int, [_VP, C.c_size_t, _VP, C.c_size_t, C.c_int, C.c_float, _VP, _VP]),
    "orc_voxel_grid": (C.c_size_t, [_VP, C.c_size_t, C.c_float, C.c_float, C.c_float, _VP, C.POINTER(C.c_int)]),
    "orc_voxel_keys": (None, [_VP, C.c_size_t, C.c_float, C.c_float, C.c_float, _VP]),
    "orc_sor": (C.c_int, [_VP, C.c_size_t, C.c_int, C.c_double, C.c_int, C.c_int, _VP, _VP, _VP]),
    "orc_normals": (C.c_int, [_VP, C.c_size_t, C.c_int, _VP, C.c_int, _VP]),
    "orc_icp": (C.c_int, [_VP, C.c_size_t, _VP, C.c_size_t, C.POINTER(IcpParams), _VP, C.POINTER(IcpResult)]),
    "orc_fitness": (C.c_double, [_VP, C.c_size_t, _VP, C.c_size_t, _VP]),
    "orc_correspondences": (C.c_int, [_VP, C.c_size_t, _VP, C.c_size_t, _VP, C.c_double, _VP, _VP]),
    "orc_crop_redundant": (C.c_size_t, [_VP, C.c_size_t, _VP, C.c_size_t, C.c_double, _VP]),
    "orc_transform": (None, [_VP, C.c_size_t, _VP, _VP]),
    "orc_centroid": (None, [_VP, C.c_size_t, _VP]),
    "orc_svd3": (None, [_VP, _VP, _VP, _VP]),
    "orc_eig3": (None, [_VP, _VP, _VP]),
    "orc_super_resolve": (None, [_VP, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, _VP, _VP,
                                 _VP]),
}

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            raise ImportError(f"{LIB} missing: run lowcost3dreconstruction_gb300.build.build_oracle()")
        _lib = C.CDLL(str(LIB))
        for name, (res, args) in _SIGS.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def _p(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


def _pts(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=POINT_DTYPE)


def set_threads(n: int) -> None:
    lib().orc_set_threads(n)


def ze_mean_u16(frames: np.ndarray) -> np.ndarray:
    frames = np.ascontiguousarray(frames, dtype=np.uint16)
    F, h, w = frames.shape
    out = np.zeros((h, w), dtype=np.uint16)
    lib().orc_ze_mean_u16(_p(frames), F, h * w, _p(out))
    return out


def ze_mean_f32(frames: np.ndarray) -> np.ndarray:
    frames = np.ascontiguousarray(frames, dtype=np.float32)
    F, h, w = frames.shape
    out = np.zeros((h, w), dtype=np.float32)
    lib().orc_ze_mean_f32(_p(frames), F, h * w, _p(out))
    return out


def image_normals_u16(depth: np.ndarray) -> np.ndarray:
    depth = np.ascontiguousarray(depth, dtype=np.uint16)
    h, w = depth.shape
    out = np.zeros((h, w, 3), dtype=np.float32)
    lib().orc_image_normals_u16(_p(depth), w, h, _p(out))
    return out


def bp_params(width, height, fx=525.0, fy=525.0, cx=319.5, cy=239.5, depth_min=0.0, depth_max=65535.0, roi=None,
              scale=1.0, normals=True, rgb=(128, 128, 128)) -> BpParams:
    l, r, t, b = roi if roi is not None else (0, width - 1, 0, height - 1)
    return BpParams(width, height, fx, fy, cx, cy, depth_min, depth_max, l, r, t, b, scale, 1 if normals else 0,
                    rgb[0], rgb[1], rgb[2], 0)


def backproject_v1(depth: np.ndarray, prm: BpParams, ascii_roundtrip: bool = False) -> np.ndarray:
    depth = np.ascontiguousarray(depth, dtype=np.uint16)
    out = np.zeros(depth.size, dtype=POINT_DTYPE)
    n = lib().orc_backproject_v1(_p(depth), C.byref(prm), 1 if ascii_roundtrip else 0, _p(out))
    return out[:n]


def backproject_v2(depth_mm: np.ndarray, prm: BpParams) -> np.ndarray:
    depth_mm = np.ascontiguousarray(depth_mm, dtype=np.float32)
    out = np.zeros(depth_mm.size, dtype=POINT_DTYPE)
    n = lib().orc_backproject_v2(_p(depth_mm), C.byref(prm), _p(out))
    return out[:n]


def knn(ref, query, k: int, max_dist_sq: float = -1.0):
    ref, query = _pts(ref), _pts(query)
    idx = np.zeros((len(query), k), dtype=np.int32)
    dist = np.zeros((len(query), k), dtype=np.float32)
    lib().orc_knn(_p(ref), len(ref), _p(query), len(query), k, max_dist_sq, _p(idx), _p(dist))
    return idx, dist


def voxel_grid(pts, leaf):
    pts = _pts(pts)
    lx, ly, lz = (leaf, leaf, leaf) if np.isscalar(leaf) else leaf
    out = np.zeros(max(len(pts), 1), dtype=POINT_DTYPE)
    ov = C.c_int(0)
    n = lib().orc_voxel_grid(_p(pts), len(pts), lx, ly, lz, _p(out), C.byref(ov))
    return out[:n], bool(ov.value)


def voxel_keys(pts, leaf) -> np.ndarray:
    pts = _pts(pts)
    keys = np.zeros(len(pts), dtype=np.int64)
    lib().orc_voxel_keys(_p(pts), len(pts), leaf, leaf, leaf, _p(keys))
    return keys


def sor(pts, mean_k: int, std_mul: float, sqrt_double: bool = False, sequential: bool = False):
    pts = _pts(pts)
    d = np.zeros(len(pts), dtype=np.float32)
    keep = np.zeros(len(pts), dtype=np.uint8)
    stats = np.zeros(4, dtype=np.float64)
    rc = lib().orc_sor(_p(pts), len(pts), mean_k, std_mul, 1 if sqrt_double else 0, 1 if sequential else 0, _p(d),
                       _p(keep), _p(stats))
    if rc != 0:
        raise ValueError(f"orc_sor failed ({rc})")
    return d, keep.astype(bool), dict(mean=stats[0], stddev=stats[1], threshold=stats[2], valid=int(stats[3]))


def normals(pts, k: int, viewpoint=(0.0, 0.0, 0.0), flip_all: bool = False) -> np.ndarray:
    pts = _pts(pts)
    vp = np.asarray(viewpoint, dtype=np.float32)
    out = np.zeros(len(pts), dtype=POINT_DTYPE)
    lib().orc_normals(_p(pts), len(pts), k, _p(vp), 1 if flip_all else 0, _p(out))
    return out


def icp(src, tgt, max_corr_dist=0.1, max_iterations=50, transformation_epsilon=1e-9, euclidean_fitness_epsilon=1e-3,
        point_to_plane=False, guess=None) -> dict:
    src, tgt = _pts(src), _pts(tgt)
    prm = IcpParams(max_corr_dist, max_iterations, transformation_epsilon, euclidean_fitness_epsilon,
                    1 if point_to_plane else 0, 3)
    res = IcpResult()
    g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float64).reshape(16)
    lib().orc_icp(_p(src), len(src), _p(tgt), len(tgt), C.byref(prm), _p(g) if g is not None else None, C.byref(res))
    return dict(transform=np.array(res.transform).reshape(4, 4), converged=bool(res.converged),
                iterations=res.iterations, state=res.state, n_corr=res.n_corr_last, fitness=res.fitness,
                mse=res.mse_last)


def correspondences(src, tgt, T, max_dist):
    src, tgt = _pts(src), _pts(tgt)
    T = np.ascontiguousarray(T, dtype=np.float64).reshape(16)
    idx = np.zeros(len(src), dtype=np.int32)
    dist = np.zeros(len(src), dtype=np.float32)
    lib().orc_correspondences(_p(src), len(src), _p(tgt), len(tgt), _p(T), max_dist, _p(idx), _p(dist))
    return idx, dist


def fitness(src, tgt, T) -> float:
    src, tgt = _pts(src), _pts(tgt)
    T = np.ascontiguousarray(T, dtype=np.float64).reshape(16)
    return float(lib().orc_fitness(_p(src), len(src), _p(tgt), len(tgt), _p(T)))


def crop_redundant(src, tgt, radius: float) -> np.ndarray:
    src, tgt = _pts(src), _pts(tgt)
    out = np.zeros(len(src), dtype=np.uint8)
    lib().orc_crop_redundant(_p(src), len(src), _p(tgt), len(tgt), radius, _p(out))
    return out.astype(bool)


def transform(pts, m) -> np.ndarray:
    pts = _pts(pts)
    m = np.ascontiguousarray(m, dtype=np.float32).reshape(16)
    out = np.zeros_like(pts)
    lib().orc_transform(_p(pts), len(pts), _p(m), _p(out))
    return out


def centroid(pts) -> np.ndarray:
    pts = _pts(pts)
    c = np.zeros(4, dtype=np.float32)
    lib().orc_centroid(_p(pts), len(pts), _p(c))
    return c


def centroid_align(src, tgt, roll=0.0, pitch=0.0, yaw=0.0, elevation=0.0, exact: bool = False):
    """centroid_align.cpp:102-130: translate the source by -c_src, rotate it by
    R = Rx(roll) Ry(pitch) Rz(yaw) (degrees, AngleAxis products in that order),
    translate by c_tgt, then by (0, elevation, 0).  exact=False restates PCL's
    float path: compute3DCentroid summed sequentially in FP32 and four
    transformPointCloudWithNormals passes with float matrices.  exact=True
    forms the centroids and the composed matrix in FP64 and applies it once.
    Returns (moved cloud, composed FP64 matrix)."""
    src, tgt = _pts(src), _pts(tgt)
    d2r = np.pi / 180.0
    a, b, c = roll * d2r, pitch * d2r, yaw * d2r
    Rx = np.array([[1, 0, 0], [0, np.cos(a), -np.sin(a)], [0, np.sin(a), np.cos(a)]])
    Ry = np.array([[np.cos(b), 0, np.sin(b)], [0, 1, 0], [-np.sin(b), 0, np.cos(b)]])
    Rz = np.array([[np.cos(c), -np.sin(c), 0], [np.sin(c), np.cos(c), 0], [0, 0, 1]])
    R = Rx @ Ry @ Rz

    def tr(t):
        m = np.eye(4)
        m[:3, 3] = t
        return m

    rot = np.eye(4)
    rot[:3, :3] = R
    if exact:
        def c64(p):
            f = np.isfinite(p["x"]) & np.isfinite(p["y"]) & np.isfinite(p["z"])
            return np.c_[p["x"][f], p["y"][f], p["z"][f]].astype(np.float64).mean(0)
        cs, ct = c64(src), c64(tgt)
    else:
        cs, ct = centroid(src)[:3].astype(np.float64), centroid(tgt)[:3].astype(np.float64)
    steps = [tr(-cs), rot, tr(ct), tr((0.0, elevation, 0.0))]
    M = steps[3] @ steps[2] @ steps[1] @ steps[0]
    if exact:
        return transform(src, M.astype(np.float32)), M
    out = src
    for m in steps:
        out = transform(out, m.astype(np.float32))
    return out, M


def svd3(a):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(9)
    u, s, v = np.zeros(9), np.zeros(3), np.zeros(9)
    lib().orc_svd3(_p(a), _p(u), _p(s), _p(v))
    return u.reshape(3, 3), s, v.reshape(3, 3)


def eig3(a):
    a = np.ascontiguousarray(a, dtype=np.float64).reshape(9)
    w, v = np.zeros(3), np.zeros(9)
    lib().orc_eig3(_p(a), _p(w), _p(v))
    return w, v.reshape(3, 3)


def super_resolve(frames: np.ndarray, factor: int = 4, iters: int = 200, eps: float = 1e-12):
    """The C restatement of the super-resolution front end (sr_oracle.cpp):
    (fused image of the frames' type, warps [F][2][3], iterations [F]);
    uint16 or float32 frames [F][h][w]."""
    f32 = np.asarray(frames).dtype == np.float32
    frames = np.ascontiguousarray(frames, dtype=np.float32 if f32 else np.uint16)
    F, h, w = frames.shape
    out = np.zeros((h, w), dtype=frames.dtype)
    warps = np.zeros((F, 6), dtype=np.float32)
    its = np.zeros(F, dtype=np.int32)
    lib().orc_super_resolve(_p(frames), int(f32), F, w, h, factor, iters, eps, _p(out), _p(warps), _p(its))
    return out, warps.reshape(F, 2, 3), its
