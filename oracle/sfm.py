"""CPU restatement of the SfM-side filters -- TEST INFRASTRUCTURE ONLY.

Used by tests/ to check lowcost3dreconstruction_gb300/csrc/sfm.cu; never by the
library.  PCL is absent, so these restate PCL's documented semantics at the
call sites in pcl_tools/crop_cloud.cpp:81-97, cluster_extraction.cpp:90-130
and planar_segmentation.cpp:80-110 (parity unpinned, like the rest of the
oracle):

* crop_box: CropBox with an identity transform, min <= p <= max inclusive,
  non-finite points in neither output.
* euclidean_clusters: components of the graph joining finite points whose
  squared FP32 distance, evaluated as FLANN does ((dx^2 + dy^2) + dz^2), is
  below float(tolerance^2); clusters in [min, max] ordered by size
  descending, equal sizes by their smallest index.
* plane_segment: the library's seeded RANSAC (the hypotheses, the FP32
  plane of three points and the inlier test are restated operation for
  operation, so the hypothesis counts agree exactly), then the FP64
  least-squares refit on the best hypothesis' inliers and the inliers again.
"""
from __future__ import annotations

import numpy as np

_M64 = (1 << 64) - 1


def _finite(xyz: np.ndarray) -> np.ndarray:
    return np.all(np.isfinite(xyz), axis=1)


def crop_box(xyz: np.ndarray, lo, hi) -> tuple[np.ndarray, np.ndarray]:
    xyz = np.asarray(xyz, np.float32)
    lo, hi = np.asarray(lo, np.float32), np.asarray(hi, np.float32)
    fin = _finite(xyz)
    with np.errstate(invalid="ignore"):
        inside = fin & np.all(xyz >= lo, axis=1) & np.all(xyz <= hi, axis=1)
    return inside, fin & ~inside


def _flann_d2(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    d = (a - b).astype(np.float32)
    return ((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]).astype(np.float32) + d[:, 2] * d[:, 2]).astype(np.float32)


def euclidean_clusters(xyz: np.ndarray, tolerance: float, min_size: int, max_size: int) -> tuple[np.ndarray, int]:
    """labels (cluster rank or -1) and the number of kept clusters."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    from scipy.spatial import cKDTree
    xyz = np.asarray(xyz, np.float32)
    n = len(xyz)
    fin = np.nonzero(_finite(xyz))[0]
    r2 = np.float32(tolerance * tolerance)
    pairs = cKDTree(xyz[fin].astype(np.float64)).query_pairs(float(tolerance) * (1 + 1e-5), output_type="ndarray")
    if len(pairs):
        a, b = fin[pairs[:, 0]], fin[pairs[:, 1]]
        keep = _flann_d2(xyz[a], xyz[b]) < r2
        a, b = a[keep], b[keep]
    else:
        a = b = np.zeros(0, np.int64)
    g = coo_matrix((np.ones(len(a)), (a, b)), shape=(n, n))
    _, comp = connected_components(g, directed=False)
    labels = np.full(n, -1, np.int64)
    sizes = np.bincount(comp[fin], minlength=comp.max() + 1 if n else 0)
    first = np.full(len(sizes), n, np.int64)
    np.minimum.at(first, comp[fin], fin)
    kept = [c for c in range(len(sizes)) if sizes[c] > 0 and min_size <= sizes[c] <= max_size]
    kept.sort(key=lambda c: (-sizes[c], first[c]))
    rank = {c: r for r, c in enumerate(kept)}
    for i in fin:
        labels[i] = rank.get(comp[i], -1)
    return labels, len(kept)


def _mix64(x: int) -> int:
    x = (x + 0x9E3779B97F4A7C15) & _M64
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & _M64
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & _M64
    return x ^ (x >> 31)


def _plane_of(p0, p1, p2) -> np.ndarray:
    f = np.float32
    ax, ay, az = f(p1[0] - p0[0]), f(p1[1] - p0[1]), f(p1[2] - p0[2])
    bx, by, bz = f(p2[0] - p0[0]), f(p2[1] - p0[1]), f(p2[2] - p0[2])
    nx = f(f(ay * bz) - f(az * by))
    ny = f(f(az * bx) - f(ax * bz))
    nz = f(f(ax * by) - f(ay * bx))
    nn = f(f(f(nx * nx) + f(ny * ny)) + f(nz * nz))
    if not (nn > 0 and np.isfinite(nn)):
        return np.array([0, 0, 0, np.inf], np.float32)
    ln = np.sqrt(nn, dtype=np.float32)
    nx, ny, nz = f(nx / ln), f(ny / ln), f(nz / ln)
    d = f(-f(f(f(nx * p0[0]) + f(ny * p0[1])) + f(nz * p0[2])))
    return np.array([nx, ny, nz, d], np.float32)


def _plane_dist(c: np.ndarray, xyz: np.ndarray) -> np.ndarray:
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    with np.errstate(invalid="ignore", over="ignore"):
        s = (c[0] * x).astype(np.float32) + (c[1] * y).astype(np.float32)
        s = s.astype(np.float32) + (c[2] * z).astype(np.float32)
        s = s.astype(np.float32) + c[3]
    return np.abs(s.astype(np.float32))


def plane_segment(xyz: np.ndarray, threshold: float, hypotheses: int, seed: int):
    """(coefficients float32[4], inlier mask, counts per hypothesis, best hypothesis)."""
    xyz = np.asarray(xyz, np.float32)
    n = len(xyz)
    t = np.float32(threshold)
    finm = _finite(xyz)
    fin = np.nonzero(finm)[0]
    if len(fin) < 3:
        return np.zeros(4, np.float32), np.zeros(n, bool), np.zeros(hypotheses, np.int64), -1
    coefs, counts = [], np.zeros(hypotheses, np.int64)
    for h in range(hypotheses):
        p = [xyz[fin[_mix64((seed ^ (h << 2) ^ j) & _M64) % len(fin)]] for j in range(3)]
        c = _plane_of(*p)
        coefs.append(c)
        with np.errstate(invalid="ignore"):
            counts[h] = int(np.sum(finm & (_plane_dist(c, xyz) < t)))
    best = int(np.argmax(counts))  # lowest index among equal counts
    c = coefs[best]
    with np.errstate(invalid="ignore"):
        inl = finm & (_plane_dist(c, xyz) < t)
    P = xyz[inl].astype(np.float64)
    if len(P) >= 3:
        m = P.mean(axis=0)
        cov = (P.T @ P) / len(P) - np.outer(m, m)
        w, v = np.linalg.eigh(cov)
        nv = v[:, 0]
        if nv @ c[:3].astype(np.float64) < 0:
            nv = -nv
        c = np.array([nv[0], nv[1], nv[2], -(nv @ m)], np.float32)
    with np.errstate(invalid="ignore"):
        inl = finm & (_plane_dist(c, xyz) < t)
    return c, inl, counts, best
