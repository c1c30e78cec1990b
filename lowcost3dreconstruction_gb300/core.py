"""Python host API over liblcr: a context owning a CUDA stream and device
clouds, and one method per C-ABI entry point.  Arrays cross as numpy arrays of
POINT_DTYPE records (the 48-byte pcl::PointXYZRGBNormal layout)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import POINT_DTYPE, LcrError


def points_from_xyz(xyz: np.ndarray, normals: np.ndarray | None = None, rgb: np.ndarray | None = None,
                    curvature: np.ndarray | None = None) -> np.ndarray:
    xyz = np.asarray(xyz, dtype=np.float32).reshape(-1, 3)
    out = np.zeros(len(xyz), dtype=POINT_DTYPE)
    out["x"], out["y"], out["z"] = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    if normals is not None:
        n = np.asarray(normals, dtype=np.float32).reshape(-1, 3)
        out["normal_x"], out["normal_y"], out["normal_z"] = n[:, 0], n[:, 1], n[:, 2]
    if rgb is not None:
        c = np.asarray(rgb, dtype=np.uint8).reshape(-1, 3)
        out["r"], out["g"], out["b"] = c[:, 0], c[:, 1], c[:, 2]
    if curvature is not None:
        out["curvature"] = np.asarray(curvature, dtype=np.float32)
    return out


def xyz_of(pts: np.ndarray) -> np.ndarray:
    return np.stack([pts["x"], pts["y"], pts["z"]], axis=1)


def normals_of(pts: np.ndarray) -> np.ndarray:
    return np.stack([pts["normal_x"], pts["normal_y"], pts["normal_z"]], axis=1)


@dataclass
class IcpOutcome:
    transform: np.ndarray      # (4, 4) float32, row-major
    transform64: np.ndarray    # (4, 4) float64
    converged: bool
    iterations: int
    state: int
    n_correspondences: int
    fitness: float
    mse: float
    status: int


class Cloud:
    """A device-resident cloud (immutable; caches its search index)."""

    def __init__(self, ctx: "Context", handle: C.c_void_p):
        self._ctx = ctx
        self.handle = handle

    def __len__(self) -> int:
        return int(self._ctx.lib.lcr_cloud_size(self.handle))

    def download(self) -> np.ndarray:
        n = len(self)
        out = np.zeros(n, dtype=POINT_DTYPE)
        self._ctx._check(self._ctx.lib.lcr_cloud_download(self._ctx.h, self.handle, L.ptr(out), n))
        return out

    def neighbours(self) -> tuple[int, np.ndarray]:
        """The neighbour rows kept by normals(..., keep_neighbours=True):
        (k, rows) with rows an (n, 32) uint32 array (lcr_cloud_neighbours)."""
        k = C.c_int(0)
        rows = np.zeros((len(self), 32), dtype=np.uint32)
        self._ctx._check(self._ctx.lib.lcr_cloud_neighbours(self._ctx.h, self.handle, C.byref(k), L.ptr(rows)))
        return k.value, rows

    def free(self) -> None:
        if self.handle and self._ctx.h:
            self._ctx.lib.lcr_cloud_free(self._ctx.h, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Context:
    """One CUDA stream on one device (lcr_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = L.load()
        h = C.c_void_p()
        st = self.lib.lcr_ctx_create(C.byref(h), device)
        if st != L.OK:
            raise LcrError(st, self.lib.lcr_status_string(st).decode())
        self.h = h

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.lcr_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ plumbing
    def _check(self, st: int, allow: tuple[int, ...] = ()) -> int:
        if st != L.OK and st not in allow:
            raise LcrError(st, self.lib.lcr_last_error(self.h).decode())
        return st

    def _cloud(self, fn, *args) -> Cloud:
        out = C.c_void_p()
        self._check(fn(self.h, *args, C.byref(out)))
        return Cloud(self, out)

    @property
    def stream(self) -> int:
        return int(self.lib.lcr_ctx_stream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(self.lib.lcr_ctx_launch_count(self.h))

    def kernel_timing(self, enable: bool) -> None:
        """Start (and reset) or stop event timing of the k-NN filter kernels."""
        self._check(self.lib.lcr_kernel_timing(self.h, 1 if enable else 0))

    def kernel_time(self, which: int) -> tuple[float, int]:
        """(summed device ms, launches) of a timed kernel since timing started."""
        ms, n = C.c_double(), C.c_uint64()
        self._check(self.lib.lcr_kernel_time(self.h, which, C.byref(ms), C.byref(n)))
        return ms.value, n.value

    def synchronize(self) -> None:
        self._check(self.lib.lcr_ctx_synchronize(self.h))

    # ------------------------------------------------------------- clouds
    def upload(self, pts: np.ndarray) -> Cloud:
        pts = np.ascontiguousarray(pts, dtype=POINT_DTYPE)
        return self._cloud(self.lib.lcr_cloud_upload, L.ptr(pts), len(pts))

    def upload_xyz(self, xyz: np.ndarray) -> Cloud:
        xyz = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
        return self._cloud(self.lib.lcr_cloud_upload_xyz, L.ptr(xyz), len(xyz))

    def from_device(self, dev_ptr: int, n: int) -> Cloud:
        return self._cloud(self.lib.lcr_cloud_from_device, C.c_void_p(dev_ptr), n)

    def concat(self, a: Cloud, b: Cloud) -> Cloud:
        return self._cloud(self.lib.lcr_cloud_concat, a.handle, b.handle)

    # ------------------------------------------------------ back-projection
    @staticmethod
    def depth_params(model: int, width: int, height: int, frames: int = 1, fx: float = 525.0, fy: float = 525.0,
                     cx: float = 319.5, cy: float = 239.5, depth_min: float = 0.0, depth_max: float = 65535.0,
                     roi: tuple[int, int, int, int] | None = None, scale: float = 1.0, normals: bool = True,
                     rgb: tuple[int, int, int] = (128, 128, 128)) -> L.DepthParams:
        left, right, top, bottom = roi if roi is not None else (0, width - 1, 0, height - 1)
        return L.DepthParams(model, width, height, frames, fx, fy, cx, cy, depth_min, depth_max, left, right, top,
                             bottom, scale, 1 if normals else 0, rgb[0], rgb[1], rgb[2], 0)

    def backproject(self, depth: np.ndarray, params: L.DepthParams) -> Cloud:
        want = np.uint16 if params.model == L.KINECT_V1 else np.float32
        depth = np.ascontiguousarray(depth, dtype=want)
        assert depth.size == params.width * params.height * params.frames
        return self._cloud(self.lib.lcr_backproject, L.ptr(depth), C.byref(params))

    def backproject_device(self, dev_ptr: int, params: L.DepthParams) -> Cloud:
        return self._cloud(self.lib.lcr_backproject_device, C.c_void_p(dev_ptr), C.byref(params))

    def backproject_into(self, dev_ptr: int, params: L.DepthParams, points_ptr: int, capacity: int,
                         count_ptr: int) -> None:
        """lcr_backproject_into: records into caller-owned device memory, the
        count into a device uint32; asynchronous on this context's stream."""
        self._check(self.lib.lcr_backproject_into(self.h, C.c_void_p(dev_ptr), C.byref(params),
                                                  C.c_void_p(points_ptr), capacity, C.c_void_p(count_ptr)))

    def burst_fuse(self, frames: np.ndarray, params: L.DepthParams) -> np.ndarray:
        want = np.uint16 if params.model == L.KINECT_V1 else np.float32
        frames = np.ascontiguousarray(frames, dtype=want)
        out = np.zeros((params.height, params.width), dtype=want)
        self._check(self.lib.lcr_burst_fuse(self.h, L.ptr(frames), C.byref(params), L.ptr(out)))
        return out

    # -------------------------------------------------------------- filters
    def voxel_grid(self, cloud: Cloud, leaf: float | tuple[float, float, float]) -> Cloud:
        lx, ly, lz = (leaf, leaf, leaf) if np.isscalar(leaf) else leaf
        return self._cloud(self.lib.lcr_voxel_grid, cloud.handle, lx, ly, lz)

    def sor(self, cloud: Cloud, mean_k: int, std_mul: float, want_outliers: bool = False):
        inl, outl = C.c_void_p(), C.c_void_p()
        stats = L.SorStats()
        self._check(self.lib.lcr_sor(self.h, cloud.handle, mean_k, std_mul, C.byref(inl),
                                     C.byref(outl) if want_outliers else None, C.byref(stats)))
        return Cloud(self, inl), (Cloud(self, outl) if want_outliers else None), stats

    def sor_distances(self, cloud: Cloud, mean_k: int) -> tuple[np.ndarray, L.SorStats]:
        out = np.zeros(len(cloud), dtype=np.float32)
        stats = L.SorStats()
        self._check(self.lib.lcr_sor_distances(self.h, cloud.handle, mean_k, L.ptr(out), C.byref(stats)))
        return out, stats

    def normals(self, cloud: Cloud, k: int, viewpoint=(0.0, 0.0, 0.0), flip_all: bool = False,
                keep_neighbours: bool = False) -> Cloud:
        """NormalEstimation (lcr_normals).  keep_neighbours (k <= 31) keeps each
        point's k nearest with the output, so that ICP with it as the target
        settles most correspondences without a search (same result)."""
        vp = np.asarray(viewpoint, dtype=np.float32)
        flags = (L.NORMALS_FLIP_ALL if flip_all else 0) | (L.NORMALS_KEEP_NEIGHBOURS if keep_neighbours else 0)
        return self._cloud(self.lib.lcr_normals, cloud.handle, k, L.ptr(vp), flags)

    # ------------------------------------------------------------------ ICP
    @staticmethod
    def icp_params(max_correspondence_distance: float = 0.1, max_iterations: int = 50,
                   transformation_epsilon: float = 1e-9, euclidean_fitness_epsilon: float = 0.001,
                   point_to_plane: bool = False, compute_fitness: bool = True, stop_iteration: int = 0,
                   stop_rms: float = 0.0) -> L.IcpParams:
        """stop_iteration / stop_rms: a pair whose RMS correspondence distance is
        still above stop_rms after stop_iteration iterations ends, not converged
        (0: off, PCL's criteria only)."""
        return L.IcpParams(max_correspondence_distance, max_iterations, transformation_epsilon,
                           euclidean_fitness_epsilon, L.ICP_POINT_TO_PLANE if point_to_plane else L.ICP_POINT_TO_POINT,
                           1 if compute_fitness else 0, stop_iteration, stop_rms)

    def icp(self, src: Cloud, tgt: Cloud, params: L.IcpParams, guess: np.ndarray | None = None,
            want_registered: bool = False):
        res = L.IcpResult()
        reg = C.c_void_p()
        g = None if guess is None else np.ascontiguousarray(guess, dtype=np.float32).reshape(16)
        st = self._check(self.lib.lcr_icp(self.h, src.handle, tgt.handle, C.byref(params),
                                          L.ptr(g) if g is not None else None, C.byref(res),
                                          C.byref(reg) if want_registered else None),
                         allow=(L.NO_CORRESPONDENCES,))
        out = IcpOutcome(np.array(res.transform, dtype=np.float32).reshape(4, 4),
                         np.array(res.transform64, dtype=np.float64).reshape(4, 4), bool(res.converged),
                         res.iterations, res.state, res.n_correspondences, res.fitness, res.mse, st)
        return (out, Cloud(self, reg)) if want_registered else out

    def icp_batch(self, srcs: list[Cloud], tgts: list[Cloud], params: L.IcpParams,
                  guesses: np.ndarray | None = None) -> list[IcpOutcome]:
        """lcr_icp_batch: pair i aligns srcs[i] onto tgts[i]; all pairs iterate together."""
        n = len(srcs)
        assert len(tgts) == n
        res = (L.IcpResult * max(n, 1))()
        hs = (C.c_void_p * max(n, 1))(*[c.handle for c in srcs])
        ht = (C.c_void_p * max(n, 1))(*[c.handle for c in tgts])
        g = None if guesses is None else np.ascontiguousarray(guesses, dtype=np.float32).reshape(n * 16)
        st = self._check(self.lib.lcr_icp_batch(self.h, hs, ht, n, C.byref(params),
                                                L.ptr(g) if g is not None else None, res),
                         allow=(L.NO_CORRESPONDENCES,))
        return [IcpOutcome(np.array(r.transform, dtype=np.float32).reshape(4, 4),
                           np.array(r.transform64, dtype=np.float64).reshape(4, 4), bool(r.converged), r.iterations,
                           r.state, r.n_correspondences, r.fitness, r.mse, st) for r in res[:n]]

    def correspondences(self, src: Cloud, tgt: Cloud, T: np.ndarray, max_dist: float):
        n = len(src)
        idx = np.zeros(n, dtype=np.int32)
        dist = np.zeros(n, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float64).reshape(16)
        self._check(self.lib.lcr_correspondences(self.h, src.handle, tgt.handle, L.ptr(T), max_dist, L.ptr(idx),
                                                 L.ptr(dist)))
        return idx, dist

    def knn(self, ref: Cloud, query: Cloud, k: int, max_dist_sq: float = -1.0):
        n = len(query)
        idx = np.zeros((n, k), dtype=np.int32)
        dist = np.zeros((n, k), dtype=np.float32)
        self._check(self.lib.lcr_knn(self.h, ref.handle, query.handle, k, max_dist_sq, L.ptr(idx), L.ptr(dist)))
        return idx, dist

    # ----------------------------------------------------------- accumulate
    def crop_redundant(self, src: Cloud, tgt: Cloud, radius: float) -> np.ndarray:
        out = np.zeros(len(src), dtype=np.uint8)
        self._check(self.lib.lcr_crop_redundant(self.h, src.handle, tgt.handle, radius, L.ptr(out)))
        return out

    def accumulate(self, src: Cloud, tgt: Cloud, radius: float = 0.05, k: int = 50, std_mul: float = 1.0,
                   all_points: bool = False):
        out, rem = C.c_void_p(), C.c_void_p()
        self._check(self.lib.lcr_accumulate(self.h, src.handle, tgt.handle, radius, k, std_mul,
                                            L.ACCUM_ALL if all_points else 0, C.byref(out), C.byref(rem)))
        return Cloud(self, out), Cloud(self, rem)

    # ------------------------------------------------- transforms, centroid
    def remove_nan(self, cloud: Cloud) -> Cloud:
        """pcl::removeNaNFromPointCloud."""
        return self._cloud(self.lib.lcr_remove_nan, cloud.handle)

    def transform(self, cloud: Cloud, m: np.ndarray) -> Cloud:
        m = np.ascontiguousarray(m, dtype=np.float32).reshape(16)
        return self._cloud(self.lib.lcr_transform, cloud.handle, L.ptr(m))

    def centroid(self, cloud: Cloud) -> np.ndarray:
        c = np.zeros(4, dtype=np.float32)
        self._check(self.lib.lcr_centroid(self.h, cloud.handle, L.ptr(c)))
        return c

    def centroid_align(self, src: Cloud, tgt: Cloud, roll=0.0, pitch=0.0, yaw=0.0, elevation=0.0):
        out = C.c_void_p()
        m = np.zeros(16, dtype=np.float32)
        self._check(self.lib.lcr_centroid_align(self.h, src.handle, tgt.handle, roll, pitch, yaw, elevation,
                                                C.byref(out), L.ptr(m)))
        return Cloud(self, out), m.reshape(4, 4)

    # ------------------------------------------------- synthetic capture pairs
    def synthetic_pairs(self, seed: int, npairs: int, points: int, yaw_deg: float = 180.0, tilt_deg: float = 20.0,
                        translation: float = 0.1, noise: bool = True) -> tuple[list[Cloud], list[Cloud], np.ndarray]:
        """lcr_synthetic_pairs: (sources, targets, exact source-to-target transforms [n][4][4])."""
        hs = (C.c_void_p * max(npairs, 1))()
        ht = (C.c_void_p * max(npairs, 1))()
        T = np.zeros((max(npairs, 1), 16), dtype=np.float32)
        p = L.SynthParams(yaw_deg, tilt_deg, translation, 1 if noise else 0)
        self._check(self.lib.lcr_synthetic_pairs(self.h, seed, npairs, points, C.byref(p), hs, ht, L.ptr(T)))
        return ([Cloud(self, C.c_void_p(hs[i])) for i in range(npairs)],
                [Cloud(self, C.c_void_p(ht[i])) for i in range(npairs)], T[:npairs].reshape(npairs, 4, 4))

    def synthetic_depth(self, seed: int, npairs: int, model: int, width: int, height: int, fx: float, fy: float,
                        cx: float, cy: float, dev_ptr: int, distance: np.ndarray | None = None,
                        points: np.ndarray | None = None, yaw_deg: float = 180.0, tilt_deg: float = 20.0,
                        translation: float = 0.1, noise: bool = True, samples_per_pixel: float = 0.0) -> np.ndarray:
        """lcr_synthetic_depth: renders the source and target views of npairs
        objects into the device buffer at dev_ptr ([2 npairs][height][width],
        uint16 mm for Kinect v1, float32 mm otherwise) at the given distances,
        or at distances that give about `points` pixels per view; returns the
        exact source-to-target transforms [n][4][4]."""
        T = np.zeros((max(npairs, 1), 16), dtype=np.float32)
        p = L.SynthParams(yaw_deg, tilt_deg, translation, 1 if noise else 0)
        cam = L.RenderParams(model, width, height, fx, fy, cx, cy, samples_per_pixel)
        d = None if distance is None else np.ascontiguousarray(distance, dtype=np.float32)
        w = None if points is None else np.ascontiguousarray(points, dtype=np.float32)
        self._check(self.lib.lcr_synthetic_depth(self.h, seed, npairs, C.byref(p), C.byref(cam),
                                                 L.ptr(d) if d is not None else None,
                                                 L.ptr(w) if w is not None else None, C.c_void_p(dev_ptr), L.ptr(T)))
        return T[:npairs].reshape(npairs, 4, 4)

    def synthetic_turntable(self, seed: int, views: int, step_deg: float, model: int, width: int, height: int,
                            fx: float, fy: float, cx: float, cy: float, dev_ptr: int, distance: float = 1.0,
                            noise: bool = True, samples_per_pixel: float = 0.0) -> np.ndarray:
        """lcr_synthetic_turntable: `views` depth images of one object turned by
        step_deg per view about its vertical axis, into the device buffer at
        dev_ptr; returns each view's object -> camera pose [views][4][4]."""
        P = np.zeros((max(views, 1), 16), dtype=np.float32)
        cam = L.RenderParams(model, width, height, fx, fy, cx, cy, samples_per_pixel)
        self._check(self.lib.lcr_synthetic_turntable(self.h, seed, views, step_deg, C.byref(cam), distance,
                                                     1 if noise else 0, C.c_void_p(dev_ptr), L.ptr(P)))
        return P[:views].reshape(views, 4, 4)

    def rmse_batch(self, clouds: list[Cloud], Ta: np.ndarray, Tb: np.ndarray) -> np.ndarray:
        """lcr_rmse_batch: RMS over each cloud's points of |Ta p - Tb p|."""
        n = len(clouds)
        a = np.ascontiguousarray(Ta, dtype=np.float64).reshape(n * 16)
        b = np.ascontiguousarray(Tb, dtype=np.float64).reshape(n * 16)
        out = np.zeros(max(n, 1), dtype=np.float64)
        hs = (C.c_void_p * max(n, 1))(*[c.handle for c in clouds])
        self._check(self.lib.lcr_rmse_batch(self.h, hs, n, L.ptr(a), L.ptr(b), L.ptr(out)))
        return out[:n]

    # ------------------------------------------------------------- autotuning
    def tune_get(self) -> dict:
        t = L.Tune()
        self._check(self.lib.lcr_tune_get(self.h, C.byref(t)))
        return {"sor_warps": t.sor_warps, "normals_warps": t.normals_warps, "icp_blocks_per_sm": t.icp_blocks_per_sm}

    def tune_set(self, sor_warps: int, normals_warps: int, icp_blocks_per_sm: int) -> None:
        t = L.Tune(sor_warps, normals_warps, icp_blocks_per_sm)
        self._check(self.lib.lcr_tune_set(self.h, C.byref(t)))

    def autotune(self, src: Cloud, tgt: Cloud, cache_path: str | None = None) -> dict:
        """lcr_autotune: times the candidate launch shapes on (src, tgt) and applies the fastest."""
        r = L.TuneReport()
        self._check(self.lib.lcr_autotune(self.h, src.handle, tgt.handle,
                                          cache_path.encode() if cache_path else None, C.byref(r)))
        ms = lambda a: {i + 1: round(a[i], 4) for i in range(8) if a[i] > 0}
        return {"sor_warps": r.chosen.sor_warps, "normals_warps": r.chosen.normals_warps,
                "icp_blocks_per_sm": r.chosen.icp_blocks_per_sm, "from_cache": bool(r.from_cache),
                "sor_ms": ms(r.sor_ms), "normals_ms": ms(r.normals_ms), "icp_ms": ms(r.icp_ms)}

    # ------------------------------------------------------- SfM-side filters
    def crop_box(self, cloud: Cloud, lo, hi) -> tuple[Cloud, Cloud]:
        """lcr_crop_box: (inside, outside) of the box [lo, hi]."""
        a = np.ascontiguousarray(lo, dtype=np.float32).reshape(3)
        b = np.ascontiguousarray(hi, dtype=np.float32).reshape(3)
        i, o = C.c_void_p(), C.c_void_p()
        self._check(self.lib.lcr_crop_box(self.h, cloud.handle, L.ptr(a), L.ptr(b), C.byref(i), C.byref(o)))
        return Cloud(self, i), Cloud(self, o)

    def euclidean_clusters(self, cloud: Cloud, tolerance: float, min_size: int = 1, max_size: int | None = None):
        """lcr_euclidean_clusters: (labels, nclusters, clustered, rest)."""
        n = len(cloud)
        labels = np.zeros(max(n, 1), dtype=np.int32)
        k = C.c_size_t()
        a, b = C.c_void_p(), C.c_void_p()
        self._check(self.lib.lcr_euclidean_clusters(self.h, cloud.handle, tolerance, min_size,
                                                    n if max_size is None else max_size, L.ptr(labels), C.byref(k),
                                                    C.byref(a), C.byref(b)))
        return labels[:n], k.value, Cloud(self, a), Cloud(self, b)

    def plane_segment(self, cloud: Cloud, threshold: float, hypotheses: int = 1024, seed: int = 0):
        """lcr_plane_segment: (coefficients, ninliers, plane, rest)."""
        coef = np.zeros(4, dtype=np.float32)
        m = C.c_size_t()
        a, b = C.c_void_p(), C.c_void_p()
        self._check(self.lib.lcr_plane_segment(self.h, cloud.handle, threshold, hypotheses, seed, L.ptr(coef),
                                               C.byref(m), C.byref(a), C.byref(b)))
        return coef, m.value, Cloud(self, a), Cloud(self, b)

    # ------------------------------------------------------ super-resolution
    def super_resolve(self, frames: np.ndarray, factor: int = 4, ecc_iterations: int = 200,
                      ecc_epsilon: float = 1e-12):
        """lcr_super_resolve (uint16 frames, Kinect v1) or lcr_super_resolve_f32
        (float32 frames, Kinect v2): (fused depth of the frames' type, warps
        [F][2][3], (min, max), iterations [F])."""
        f32 = np.asarray(frames).dtype == np.float32
        dt = np.float32 if f32 else np.uint16
        frames = np.ascontiguousarray(frames, dtype=dt)
        F, h, w = frames.shape
        out = np.zeros((h, w), dtype=dt)
        warps = np.zeros((F, 6), dtype=np.float32)
        mm = np.zeros(2, dtype=np.float32)
        it = np.zeros(F, dtype=np.int32)
        p = L.SrParams(w, h, F, factor, ecc_iterations, ecc_epsilon)
        fn = self.lib.lcr_super_resolve_f32 if f32 else self.lib.lcr_super_resolve
        self._check(fn(self.h, L.ptr(frames), C.byref(p), L.ptr(out), L.ptr(warps), L.ptr(mm), L.ptr(it)))
        return out, warps.reshape(F, 2, 3), (float(mm[0]), float(mm[1])), it
