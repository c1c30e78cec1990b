"""CPU checks of the oracle itself against independent known answers: scipy's
kd-tree, numpy's FP64 linear algebra, brute force, and closed-form geometry.
The reference ships no tests or golden vectors, so these (with the fixtures
under tests/golden/) are what the oracle is checked against."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_cloud
from lowcost3dreconstruction_gb300.core import points_from_xyz, xyz_of, normals_of
from oracle import oracle as O


def flann_d2(q: np.ndarray, p: np.ndarray) -> np.ndarray:
    """FLANN L2_Simple<float> on 3 components: ((d0*d0) + d1*d1) + d2*d2 in float32."""
    d = (q[:, None, :].astype(np.float32) - p[None, :, :].astype(np.float32)).astype(np.float32)
    s = (d[..., 0] * d[..., 0]).astype(np.float32)
    s = (s + (d[..., 1] * d[..., 1]).astype(np.float32)).astype(np.float32)
    return (s + (d[..., 2] * d[..., 2]).astype(np.float32)).astype(np.float32)


def brute_knn(ref: np.ndarray, qry: np.ndarray, k: int):
    d = flann_d2(xyz_of(qry), xyz_of(ref))
    idx = np.lexsort((np.broadcast_to(np.arange(d.shape[1]), d.shape), d), axis=1)[:, :k]
    return idx.astype(np.int32), np.take_along_axis(d, idx, axis=1)


# ------------------------------------------------------------------ kNN
@pytest.mark.parametrize("n,m,k,lat", [(500, 200, 1, 0.0), (700, 300, 8, 0.0), (400, 150, 30, 0.05),
                                       (300, 100, 51, 0.1)])
def test_knn_matches_brute_force_with_lowest_index_ties(n, m, k, lat):
    ref = random_cloud(n, 1, lattice=lat, dup_frac=0.05)
    qry = random_cloud(m, 2, lattice=lat)
    oi, od = O.knn(ref, qry, k)
    bi, bd = brute_knn(ref, qry, k)
    np.testing.assert_array_equal(od.view(np.uint32), bd.view(np.uint32))
    np.testing.assert_array_equal(oi, bi)


def test_knn_distances_match_scipy():
    spatial = pytest.importorskip("scipy.spatial")
    ref = random_cloud(3000, 3)
    qry = random_cloud(1000, 4)
    _, od = O.knn(ref, qry, 10)
    sd, _ = spatial.cKDTree(xyz_of(ref).astype(np.float64)).query(xyz_of(qry).astype(np.float64), 10)
    np.testing.assert_allclose(od.astype(np.float64), sd ** 2, rtol=1e-5, atol=1e-9)


def test_knn_cap_and_missing_entries():
    ref = random_cloud(50, 5)
    qry = random_cloud(20, 6)
    oi, od = O.knn(ref, qry, 5, max_dist_sq=0.05)
    bi, bd = brute_knn(ref, qry, 5)
    keep = bd <= np.float32(0.05)
    np.testing.assert_array_equal(np.where(keep, bi, -1), oi)
    assert np.all(np.isinf(od[~keep]))


# ------------------------------------------------------------ voxel grid
def test_voxel_grid_lattice_known_answer():
    # two points per 1 cm voxel, symmetric about its centre: the centroid is the centre
    c = (np.stack(np.meshgrid(np.arange(4), np.arange(3), np.arange(2), indexing="ij"), -1).reshape(-1, 3) + 0.5) * 0.01
    off = np.array([0.002, -0.001, 0.0015])
    pts = points_from_xyz(np.concatenate([c + off, c - off]).astype(np.float32))
    out, overflow = O.voxel_grid(pts, 0.01)
    assert not overflow and len(out) == len(c)
    # ascending voxel index: x fastest, then y, then z
    want = c[np.lexsort((np.floor(c[:, 0] / 0.01), np.floor(c[:, 1] / 0.01), np.floor(c[:, 2] / 0.01)))]
    np.testing.assert_allclose(xyz_of(out), want, atol=1e-6)


def test_voxel_grid_overflow_returns_input():
    pts = random_cloud(100, 7, scale=1000.0)
    out, overflow = O.voxel_grid(pts, 1e-4)
    assert overflow and len(out) == len(pts)


# ------------------------------------------------------------------ SOR
def sor_brute(pts: np.ndarray, k: int, mul: float):
    _, d = brute_knn(pts, pts, k + 1)
    dist = np.empty(len(pts), np.float32)
    for i in range(len(pts)):
        s = 0.0
        for j in range(1, k + 1):  # ascending, double, float sqrt
            s += float(np.sqrt(np.float32(d[i, j])))
        dist[i] = np.float32(s / k)
    return dist


def test_sor_distances_match_brute_force():
    pts = random_cloud(600, 8, scale=0.1)
    od, keep, st = O.sor(pts, 10, 1.0)
    np.testing.assert_array_equal(od.view(np.uint32), sor_brute(pts, 10, 1.0).view(np.uint32))
    # PCL's one-pass form: sum and sum of float squares in double
    v = od.astype(np.float64)
    s, sq, n = v.sum(), (od * od).astype(np.float64).sum(), len(v)
    assert st["mean"] == pytest.approx(s / n, rel=1e-12)
    assert st["stddev"] == pytest.approx(np.sqrt((sq - s * s / n) / (n - 1)), rel=1e-9)
    np.testing.assert_array_equal(keep, od.astype(np.float64) <= st["threshold"])


def test_sor_far_point_removed_and_too_few_points():
    pts = random_cloud(300, 9, scale=0.05)
    pts["x"][17] = 5.0
    _, keep, _ = O.sor(pts, 8, 2.0)
    assert not keep[17] and keep.sum() >= 290
    with pytest.raises(ValueError):
        O.sor(random_cloud(5, 10), 5, 1.0)


def test_sor_sqrt_in_double_changes_low_bits_only():
    pts = random_cloud(800, 11, scale=0.2)
    a, _, _ = O.sor(pts, 20, 1.0)
    b, _, _ = O.sor(pts, 20, 1.0, sqrt_double=True)
    np.testing.assert_allclose(a, b, rtol=1e-6)


# -------------------------------------------------------------- normals
def test_normals_of_a_tilted_plane():
    rng = np.random.default_rng(12)
    n = np.array([0.3, -0.2, 0.93])
    n /= np.linalg.norm(n)
    a = np.cross(n, [1.0, 0, 0]); a /= np.linalg.norm(a)
    b = np.cross(n, a)
    uv = rng.uniform(-0.05, 0.05, (1500, 2))
    p = uv[:, :1] * a + uv[:, 1:] * b + np.array([0.0, 0.0, -0.8])
    out = O.normals(points_from_xyz(p), 20)
    got = normals_of(out).astype(np.float64)
    assert np.min(np.abs(got @ n)) > 1 - 1e-6
    assert np.all(np.sum(-p * got, axis=1) >= 0)          # faces the origin viewpoint
    assert np.max(out["curvature"]) < 1e-6


def test_normals_flip_all_and_few_neighbours():
    p = points_from_xyz(np.array([[0, 0, -1], [0.01, 0, -1], [0, 0.01, -1], [0.01, 0.01, -1.001]], np.float32))
    a = normals_of(O.normals(p, 4))
    b = normals_of(O.normals(p, 4, flip_all=True))
    np.testing.assert_allclose(a, -b)
    two = O.normals(p[:2], 4)  # fewer than 3 neighbours: NaN
    assert np.all(np.isnan(normals_of(two)))


# -------------------------------------------------------------- FP64 linear algebra
def test_svd3_and_eig3_match_numpy():
    rng = np.random.default_rng(13)
    for _ in range(50):
        A = rng.normal(size=(3, 3))
        U, s, V = O.svd3(A)
        np.testing.assert_allclose(s, np.linalg.svd(A, compute_uv=False), rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(U @ np.diag(s) @ V.T, A, atol=1e-12)
        S = A @ A.T
        w, E = O.eig3(S)
        np.testing.assert_allclose(w, np.linalg.eigvalsh(S), rtol=1e-10, atol=1e-12)
        np.testing.assert_allclose(S @ E, E * w, atol=1e-10)


# ------------------------------------------------------------------ ICP
def _rigid(deg: float, t) -> np.ndarray:
    a = np.deg2rad(deg)
    T = np.eye(4)
    T[:3, :3] = [[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]]
    T[:3, 3] = t
    return T


def test_icp_exact_copy_is_identity():
    pts = random_cloud(2000, 14, scale=0.1)
    r = O.icp(pts, pts, max_corr_dist=0.05, max_iterations=10, transformation_epsilon=1e-12)
    np.testing.assert_allclose(r["transform"], np.eye(4), atol=1e-6)
    assert r["converged"] and r["fitness"] == 0.0


def test_icp_recovers_a_small_rigid_motion():
    rng = np.random.default_rng(15)
    xyz = rng.uniform(-0.1, 0.1, (3000, 3))
    xyz[:, 2] += 0.3 * np.sin(8 * xyz[:, 0]) * np.cos(6 * xyz[:, 1])  # curved surface: well conditioned
    T = _rigid(3.0, (0.004, -0.002, 0.003))
    src = points_from_xyz(xyz)
    tgt = points_from_xyz((xyz @ T[:3, :3].T) + T[:3, 3])
    r = O.icp(src, tgt, max_corr_dist=0.05, max_iterations=100, transformation_epsilon=1e-12,
              euclidean_fitness_epsilon=1e-12)
    np.testing.assert_allclose(r["transform"], T, atol=2e-4)


def test_icp_no_correspondences():
    a = random_cloud(100, 16, scale=0.01)
    b = random_cloud(100, 17, scale=0.01)
    b["x"] += 10.0
    r = O.icp(a, b, max_corr_dist=0.1)
    assert not r["converged"]
    np.testing.assert_allclose(r["transform"], np.eye(4))


# ----------------------------------------------------- depth and crop
def test_backproject_constant_depth_plane():
    depth = np.full((48, 64), 1000, np.uint16)
    depth[0, 0] = 0
    prm = O.bp_params(64, 48, fx=50.0, fy=50.0, cx=31.5, cy=23.5, scale=0.001, normals=True)
    out = O.backproject_v1(depth, prm)
    assert len(out) == 64 * 48 - 1
    xyz = xyz_of(out).astype(np.float64)
    np.testing.assert_allclose(xyz[:, 2], -1.0, atol=1e-7)
    i, j = np.divmod(np.arange(1, 64 * 48), 64)
    np.testing.assert_allclose(xyz[:, 0], (j - 31.5) / 50.0, atol=1e-6)
    np.testing.assert_allclose(xyz[:, 1], -(i - 23.5) / 50.0, atol=1e-6)
    inner = (i > 1) & (i < 46) & (j > 1) & (j < 62)
    np.testing.assert_allclose(normals_of(out)[inner], [[0, 0, 1]] * int(inner.sum()), atol=1e-7)


def test_ze_mean_ignores_zeros_and_rounds_half_even():
    f = np.zeros((4, 2, 3), np.uint16)
    f[:, 0, 0] = [0, 0, 0, 0]        # no sample -> 0
    f[:, 0, 1] = [10, 0, 11, 0]      # 10.5 -> 10 (half to even)
    f[:, 0, 2] = [11, 12, 0, 0]      # 11.5 -> 12
    f[:, 1, 0] = [65535, 65535, 0, 0]
    f[:, 1, 1] = [1, 2, 2, 0]        # 1.666.. -> 2
    f[:, 1, 2] = [7, 0, 0, 0]
    np.testing.assert_array_equal(O.ze_mean_u16(f), [[0, 10, 12], [65535, 2, 7]])


def test_crop_matches_brute_force():
    src = random_cloud(400, 18, scale=0.1)
    tgt = random_cloud(300, 19, scale=0.1)
    r = 0.01
    got = O.crop_redundant(src, tgt, r)
    s, t = xyz_of(src), xyz_of(tgt)
    lo = (t.astype(np.float64) - r).astype(np.float32)
    hi = (t.astype(np.float64) + r).astype(np.float32)
    inside = np.all((s[:, None, :] >= lo[None]) & (s[:, None, :] <= hi[None]), axis=2).any(axis=1)
    np.testing.assert_array_equal(got, inside)
