"""GPU parity: every kernel of the alignment path against the CPU oracle on the
same seeded inputs, through the C ABI.

Bar: bit-exact for neighbour indices/distances, voxel membership and
centroids (shared summation order), back-projection, burst fusion, SOR mean
distances and masks, crop masks; FP64-oracle tolerances for normals
(angle <= 1e-3 rad away from near-degenerate spectra) and ICP transforms
(1e-5 rad rotation, 1e-6 x cloud extent translation)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import random_cloud
from lowcost3dreconstruction_gb300 import _lib as L
from lowcost3dreconstruction_gb300 import synthetic as S
from lowcost3dreconstruction_gb300.core import xyz_of, normals_of
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _extent(pts) -> float:
    x = xyz_of(pts)
    return float(np.max(x.max(0) - x.min(0)))


def _rot_angle(Ra, Rb) -> float:
    R = np.asarray(Ra, np.float64)[:3, :3] @ np.asarray(Rb, np.float64)[:3, :3].T
    return float(np.arccos(np.clip((np.trace(R) - 1) / 2, -1, 1)))


def _assert_transform_close(Ta, Tb, extent, rot_tol=1e-5, trans_rel=1e-6, at=None):
    """Rotation angle between the two transforms, and the translation they give
    the cloud: the displacement of the point `at` (the source centroid), since a
    rotation difference moves the origin-referenced translation by the lever arm
    to the cloud (~1 m here)."""
    assert _rot_angle(Ta, Tb) <= rot_tol, _rot_angle(Ta, Tb)
    p = np.r_[np.zeros(3) if at is None else np.asarray(at, np.float64), 1.0]
    dt = np.linalg.norm((np.asarray(Ta, np.float64) - np.asarray(Tb, np.float64)) @ p)
    assert dt <= trans_rel * extent, (dt, extent)


def _centroid(pts):
    return xyz_of(pts).astype(np.float64).mean(0)


# ------------------------------------------------------------------ kNN
@pytest.mark.parametrize("n,m,k,seed,lat,dup", [
    (1, 1, 1, 0, 0.0, 0.0), (33, 7, 1, 1, 0.0, 0.0), (5000, 3000, 1, 2, 0.0, 0.0),
    (20000, 20000, 1, 3, 0.05, 0.1), (4000, 4000, 8, 4, 0.0, 0.0), (6000, 5000, 51, 5, 0.1, 0.05),
    (3000, 2000, 30, 6, 0.0, 0.0), (100, 64, 100, 7, 0.0, 0.0)])
def test_knn_bit_exact(ctx, n, m, k, seed, lat, dup):
    ref = random_cloud(n, seed, lattice=lat, dup_frac=dup)
    qry = random_cloud(m, seed + 100, lattice=lat)
    gi, gd = ctx.knn(ctx.upload(ref), ctx.upload(qry), k)
    oi, od = O.knn(ref, qry, k)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gd.view(np.uint32), od.view(np.uint32))


def test_knn_capped_and_self(ctx, cfg0):
    t = cfg0["vtgt"]
    c = ctx.upload(t)
    for cap in (1e-6, 4e-6, 2.5e-3):
        gi, gd = ctx.knn(c, c, 4, cap)
        oi, od = O.knn(t, t, 4, cap)
        np.testing.assert_array_equal(gi, oi)
        np.testing.assert_array_equal(gd, od)


def test_knn_nonfinite_points(ctx):
    ref = random_cloud(500, 11)
    qry = random_cloud(300, 12)
    ref["x"][::7] = np.nan
    qry["y"][::5] = np.inf
    gi, gd = ctx.knn(ctx.upload(ref), ctx.upload(qry), 3)
    oi, od = O.knn(ref, qry, 3)
    np.testing.assert_array_equal(gi, oi)
    np.testing.assert_array_equal(gd, od)


def test_correspondences_bit_exact(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    cs, ct = ctx.upload(s), ctx.upload(t)
    for T in (np.eye(4), cfg0["pair"].T_gt, S.turntable(7.0, S.OBJECT_AXIS, (0.01, 0.0, 0.0))):
        for dmax in (0.005, 0.05):
            gi, gd = ctx.correspondences(cs, ct, T, dmax)
            oi, od = O.correspondences(s, t, T, dmax)
            np.testing.assert_array_equal(gi, oi)
            np.testing.assert_array_equal(gd, od)


# ------------------------------------------------------ depth -> cloud
def test_burst_fuse_u16_bit_exact(ctx):
    pr = S.config1_pair(1)
    p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=10)
    np.testing.assert_array_equal(ctx.burst_fuse(pr.src_frames, p), O.ze_mean_u16(pr.src_frames))


def test_burst_fuse_f32_bit_exact(ctx):
    rng = np.random.default_rng(3)
    fr = rng.uniform(500, 3000, size=(7, 424, 512)).astype(np.float32)
    fr[rng.random(fr.shape) < 0.3] = 0
    fr[:, :10, :10] = 0
    p = ctx.depth_params(L.KINECT_V2, 512, 424, frames=7)
    np.testing.assert_array_equal(ctx.burst_fuse(fr, p), O.ze_mean_f32(fr))


def _cmp_points(g, o, fields=("x", "y", "z", "normal_x", "normal_y", "normal_z", "curvature", "r", "g", "b")):
    assert len(g) == len(o)
    for f in fields:
        a, b = g[f], o[f]
        if a.dtype.kind == "f":
            np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32), err_msg=f)
        else:
            np.testing.assert_array_equal(a, b, err_msg=f)


@pytest.mark.parametrize("scale,roi,drange", [(1.0, None, (0, 65535)), (0.001, (40, 600, 30, 450), (900, 1200)),
                                              (0.01, None, (0, 65535))])
def test_backproject_v1_bit_exact(ctx, cfg0, scale, roi, drange):
    depth = cfg0["pair"].src_frames[0]
    p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=1, depth_min=drange[0], depth_max=drange[1], roi=roi,
                         scale=scale, normals=True)
    g = ctx.backproject(depth, p).download()
    o = O.backproject_v1(depth, O.bp_params(640, 480, depth_min=drange[0], depth_max=drange[1], roi=roi,
                                            scale=scale, normals=True))
    _cmp_points(g, o)


def test_backproject_v1_burst_bit_exact(ctx):
    pr = S.config1_pair(1)
    p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=10, scale=0.001, depth_max=4000)
    g = ctx.backproject(pr.src_frames, p).download()
    o = O.backproject_v1(O.ze_mean_u16(pr.src_frames), O.bp_params(640, 480, scale=0.001, depth_max=4000))
    _cmp_points(g, o)
    assert len(g) > 250_000


def test_backproject_v2_bit_exact(ctx):
    cam = S.KINECT_V2
    d = S.raycast(S.sphere_on_cube_room(), cam)
    fr = S.kinect_frames(d, 1, np.random.default_rng(4), as_float=True)
    fr[0, 5, 5] = np.nan
    p = ctx.depth_params(L.KINECT_V2, 512, 424, fx=365.0, fy=365.0, cx=255.5, cy=211.5, depth_min=500,
                         depth_max=2500, roi=(20, 490, 10, 400), scale=1000.0 / 4500.0, normals=False)
    g = ctx.backproject(fr, p).download()
    o = O.backproject_v2(fr[0], O.bp_params(512, 424, fx=365.0, fy=365.0, cx=255.5, cy=211.5, depth_min=500,
                                            depth_max=2500, roi=(20, 490, 10, 400), scale=1000.0 / 4500.0,
                                            normals=False))
    _cmp_points(g, o, fields=("x", "y", "z"))


# ------------------------------------------------------------ voxel grid
@pytest.mark.parametrize("leaf", [0.001, 0.002, 0.0075])
def test_voxel_grid_bit_exact(ctx, cfg0, leaf):
    pts = cfg0["src"]
    g = ctx.voxel_grid(ctx.upload(pts), leaf).download()
    o, ov = O.voxel_grid(pts, leaf)
    assert not ov
    _cmp_points(g, o)


def test_voxel_grid_random_rgb(ctx):
    pts = random_cloud(50000, 21, scale=0.2)
    g = ctx.voxel_grid(ctx.upload(pts), 0.03).download()
    o, _ = O.voxel_grid(pts, 0.03)
    _cmp_points(g, o)


def test_voxel_grid_overflow_returns_input(ctx):
    pts = random_cloud(1000, 22, scale=100.0)
    g = ctx.voxel_grid(ctx.upload(pts), 1e-4).download()
    o, ov = O.voxel_grid(pts, 1e-4)
    assert ov and len(g) == len(pts)
    _cmp_points(g, o, fields=("x", "y", "z"))


# ------------------------------------------------------------------ SOR
@pytest.mark.parametrize("k,mul", [(50, 1.0), (50, 5.0), (10, 0.5)])
def test_sor_bit_exact(ctx, cfg0, k, mul):
    pts = cfg0["vsrc"]
    c = ctx.upload(pts)
    gd, gs = ctx.sor_distances(c, k)
    od, okeep, ost = O.sor(pts, k, mul)
    np.testing.assert_array_equal(gd.view(np.uint32), od.view(np.uint32))
    inl, outl, st = ctx.sor(c, k, mul, want_outliers=True)
    assert st.threshold == ost["threshold"] and st.mean == ost["mean"] and st.stddev == ost["stddev"]
    assert st.kept == int(okeep.sum()) and st.removed == int((~okeep).sum())
    _cmp_points(inl.download(), pts[okeep])
    _cmp_points(outl.download(), pts[~okeep])


def _stacked_duplicates(seed: int) -> np.ndarray:
    """A cloud where 80 copies of 3 points make the k-th neighbour of their
    neighbourhoods fall among dozens of equal distances (the boundary of the
    unordered k-NN form is then split on the index part of the key)."""
    pts = random_cloud(3000, seed, scale=0.05)
    return np.concatenate([pts] + [pts[[7, 1500, 2999]]] * 80)


def _dynamic_range_cloud(seed: int) -> np.ndarray:
    """Neighbour distances 1e-10 beside ~1e-2: the double sum of the SOR mean
    can round, so only the ascending order gives the reference's value (those
    tiles take the sorted form)."""
    pts = random_cloud(2000, seed, scale=0.05)
    near = pts[:40].copy()
    near["x"] = np.float32(0.0)
    near["y"] = np.float32(0.0)
    near["z"] = (np.arange(40) * 1e-10).astype(np.float32)
    return np.concatenate([pts, near])


@pytest.mark.parametrize("make", [_stacked_duplicates, _dynamic_range_cloud])
def test_sor_ties_and_dynamic_range_bit_exact(ctx, make):
    pts = make(3)
    gd, _ = ctx.sor_distances(ctx.upload(pts), 50)
    od, _, _ = O.sor(pts, 50, 1.0)
    np.testing.assert_array_equal(gd.view(np.uint32), od.view(np.uint32))


def _eigengap(pts, k):
    """(l1 - l0) / trace of each point's k-neighbourhood covariance (FP64)."""
    idx, _ = O.knn(pts, pts, k)
    x = xyz_of(pts).astype(np.float64)[idx]
    d = x - x.mean(1, keepdims=True)
    w = np.linalg.eigvalsh(np.einsum("nki,nkj->nij", d, d) / k)
    tr = w.sum(1)
    return np.where(tr > 0, (w[:, 1] - w[:, 0]) / np.where(tr > 0, tr, 1), 0.0)


def test_normals_coincident_points(ctx):
    pts = _stacked_duplicates(4)
    g = ctx.normals(ctx.upload(pts), 30).download()
    o = O.normals(pts, 30)
    ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
    # coincident neighbourhoods: NaN normal, curvature 0 on both sides
    zero = ~np.isfinite(no[:, 0])
    assert zero.sum() >= 240
    assert np.all(~np.isfinite(ng[zero, 0])) and np.all(g["curvature"][zero] == 0)
    # elsewhere the normal is defined where the smallest eigenvalue is simple
    ok = ~zero & (o["curvature"] < 0.2) & (_eigengap(pts, 30) > 1e-3)
    ang = np.arccos(np.clip(np.abs(np.sum(ng * no, axis=1)[ok]), -1, 1))
    assert np.percentile(ang, 99.9) < 1e-3
    np.testing.assert_allclose(g["curvature"][ok], o["curvature"][ok], atol=1e-4)


def test_sor_far_point_removed(ctx):
    pts = random_cloud(2000, 31, scale=0.1)
    pts["x"][1234] = 10.0
    inl, _, st = ctx.sor(ctx.upload(pts), 20, 3.0)
    out = inl.download()
    assert st.removed >= 1 and not np.any(out["x"] == 10.0)


def test_sor_too_few_points(ctx):
    pts = random_cloud(10, 32)
    with pytest.raises(L.LcrError) as e:
        ctx.sor(ctx.upload(pts), 10, 1.0)
    assert e.value.status == L.TOO_FEW_POINTS


# -------------------------------------------------------------- normals
def _normal_agreement(g, o, k):
    ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
    cos = np.abs(np.sum(ng * no, axis=1))
    return cos, np.sum(ng * no, axis=1)


@pytest.mark.parametrize("k", [30, 50])
def test_normals_vs_fp64_oracle(ctx, cfg0, k):
    pts = cfg0["vsrc"]
    g = ctx.normals(ctx.upload(pts), k).download()
    o = O.normals(pts, k)
    _cmp_points(g, o, fields=("x", "y", "z", "r", "g", "b"))
    ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
    dot = np.sum(ng * no, axis=1)
    ok = o["curvature"] < 0.2  # away from near-isotropic neighbourhoods
    ang = np.arccos(np.clip(np.abs(dot[ok]), -1, 1))
    assert np.percentile(ang, 99.9) < 1e-3, np.percentile(ang, 99.9)
    assert np.mean(dot[ok] > 0) > 0.999  # same viewpoint orientation
    np.testing.assert_allclose(g["curvature"][ok], o["curvature"][ok], atol=1e-4)


@pytest.mark.parametrize("k", [30, 51])
def test_normals_of_sor_inliers_from_neighbour_lists(ctx, cfg0, k):
    # SOR hands its exact 51-NN lists to the inliers; normals select from them
    # (k=51 leaves every point with an outlier in its list to the search)
    pts = cfg0["vsrc"]
    inl, _, _ = ctx.sor(ctx.upload(pts), 50, 1.0)
    g = ctx.normals(inl, k).download()
    _, okeep, _ = O.sor(pts, 50, 1.0)
    o = O.normals(pts[okeep], k)
    _cmp_points(g, o, fields=("x", "y", "z", "r", "g", "b"))
    ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
    dot = np.sum(ng * no, axis=1)
    ok = o["curvature"] < 0.2
    ang = np.arccos(np.clip(np.abs(dot[ok]), -1, 1))
    assert np.percentile(ang, 99.9) < 1e-3, np.percentile(ang, 99.9)
    assert np.mean(dot[ok] > 0) > 0.999
    np.testing.assert_allclose(g["curvature"][ok], o["curvature"][ok], atol=1e-4)
    # the same cloud without the lists (searched): same neighbours, FP32 sums in
    # another order -- agreement at the normals' FP32 bar
    s = ctx.normals(ctx.upload(inl.download()), k).download()
    cos = np.abs(np.sum(normals_of(s).astype(np.float64) * ng, axis=1))
    assert np.percentile(np.arccos(np.clip(cos[ok], -1, 1)), 99.9) < 1e-3


def test_normals_of_sor_inliers_without_usable_lists(ctx, cfg0):
    # SOR k=10 hands lists of 11 keys: they cannot serve normals k=30 (searched),
    # they serve k=8 once (consumed), and a second k=8 call searches
    pts = cfg0["vsrc"]
    inl, _, _ = ctx.sor(ctx.upload(pts), 10, 1.0)
    _, okeep, _ = O.sor(pts, 10, 1.0)

    def check(g, k):
        o = O.normals(pts[okeep], k)
        ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
        ok = o["curvature"] < 0.2
        ang = np.arccos(np.clip(np.abs(np.sum(ng * no, axis=1)[ok]), -1, 1))
        assert np.percentile(ang, 99.9) < 1e-3, (k, np.percentile(ang, 99.9))

    check(ctx.normals(inl, 30).download(), 30)
    listed = ctx.normals(inl, 8).download()
    searched = ctx.normals(inl, 8).download()
    check(listed, 8)
    check(searched, 8)


def test_normals_plane_known_answer(ctx):
    rng = np.random.default_rng(5)
    xy = rng.uniform(-0.1, 0.1, size=(4000, 2))
    n = np.array([0.2, -0.3, 0.9])
    n /= np.linalg.norm(n)
    a = np.cross(n, [1, 0, 0]); a /= np.linalg.norm(a)
    b = np.cross(n, a)
    p = xy[:, :1] * a + xy[:, 1:] * b + np.array([0.0, 0.0, -1.0])
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    g = ctx.normals(ctx.upload(points_from_xyz(p)), 20).download()
    ng = normals_of(g).astype(np.float64)
    assert np.min(np.abs(ng @ n)) > 1 - 1e-5
    # viewpoint (origin) side: (vp - p).n >= 0
    assert np.all(np.sum((-p) * ng, axis=1) >= -1e-6)
    assert np.max(g["curvature"]) < 1e-5


# ------------------------------------------------------------------ ICP
def test_icp_p2p_matches_oracle(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=50, transformation_epsilon=1e-8)
    g = ctx.icp(ctx.upload(s), ctx.upload(t), prm)
    o = O.icp(s, t, max_corr_dist=0.05, max_iterations=50, transformation_epsilon=1e-8)
    assert g.converged == o["converged"]
    assert abs(g.iterations - o["iterations"]) <= 1
    _assert_transform_close(g.transform64, o["transform"], _extent(s), at=_centroid(s))
    assert abs(g.fitness - o["fitness"]) <= 1e-4 * o["fitness"]
    # The end point of this slowly creeping trajectory (the sphere is symmetric
    # about the motion axis) moves by more than the GPU-oracle gap when the
    # oracle itself starts 1e-7 rad away: the gap is round-off, amplified.
    Gp = S.rigid(S.rot_y(np.rad2deg(1e-7)), (0.0, 0.0, 0.0))
    o2 = O.icp(s, t, max_corr_dist=0.05, max_iterations=50, transformation_epsilon=1e-8, guess=Gp)
    spread = _rot_angle(o2["transform"], o["transform"])
    assert _rot_angle(g.transform64, o["transform"]) <= max(spread, 1e-6)


def test_icp_p2plane_matches_oracle_and_ground_truth(ctx, cfg0):
    s = O.normals(cfg0["vsrc"], 30)
    t = O.normals(cfg0["vtgt"], 30)
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=50, transformation_epsilon=1e-8,
                         point_to_plane=True)
    g = ctx.icp(ctx.upload(s), ctx.upload(t), prm)
    o = O.icp(s, t, max_corr_dist=0.05, max_iterations=50, transformation_epsilon=1e-8, point_to_plane=True)
    assert g.converged and o["converged"]
    assert abs(g.iterations - o["iterations"]) <= 1
    _assert_transform_close(g.transform64, o["transform"], _extent(s), at=_centroid(s))
    assert S.rmse(g.transform64, cfg0["pair"].T_gt, xyz_of(s)) < 1e-3


@pytest.mark.parametrize("p2pl", [False, True])
def test_icp_single_iteration_matches_oracle(ctx, cfg0, p2pl):
    """One iteration from the same state: the GPU increment (FP32 terms, Kahan +
    FP64 reduction, FP64 solve) equals the FP64 oracle's to 1e-6 rad / 1e-6 x extent."""
    s = O.normals(cfg0["vsrc"], 30) if p2pl else cfg0["vsrc"]
    t = O.normals(cfg0["vtgt"], 30) if p2pl else cfg0["vtgt"]
    cs, ct = ctx.upload(s), ctx.upload(t)
    for T0 in (np.eye(4), cfg0["pair"].T_gt, S.turntable(10.0, S.OBJECT_AXIS, (0.01, 0.0, 0.0))):
        guess = T0.astype(np.float32)
        prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=1, point_to_plane=p2pl)
        g = ctx.icp(cs, ct, prm, guess=guess)
        o = O.icp(s, t, max_corr_dist=0.05, max_iterations=1, point_to_plane=p2pl, guess=guess)
        assert g.iterations == o["iterations"] == 1 and g.n_correspondences == o["n_corr"]
        assert abs(g.mse - o["mse"]) <= 1e-6 * o["mse"]
        _assert_transform_close(g.transform64, o["transform"], _extent(s), rot_tol=1e-6, at=_centroid(s))


@pytest.mark.parametrize("p2pl", [False, True])
def test_icp_exact_rigid_copy(ctx, cfg0, p2pl):
    """Known answer: a noiseless rigid copy is registered to FP32 round-off of
    the copy (measured: 0 rad, <= 5e-8 x extent), by both implementations."""
    s = O.normals(cfg0["vsrc"], 30)
    R = S.rot_x(2.0) @ S.rot_y(-3.0)
    T = S.rigid(R, (0.004, -0.002, 0.003))
    t = O.transform(s, T.astype(np.float32))
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=100, transformation_epsilon=1e-12,
                         euclidean_fitness_epsilon=1e-12, point_to_plane=p2pl)
    g = ctx.icp(ctx.upload(s), ctx.upload(t), prm)
    _assert_transform_close(g.transform64, T, _extent(s), rot_tol=1e-6, trans_rel=1e-6, at=_centroid(s))
    o = O.icp(s, t, max_corr_dist=0.05, max_iterations=100, transformation_epsilon=1e-12,
              euclidean_fitness_epsilon=1e-12, point_to_plane=p2pl)
    _assert_transform_close(g.transform64, o["transform"], _extent(s), rot_tol=1e-6, trans_rel=1e-6,
                            at=_centroid(s))


def test_icp_no_correspondences(ctx, cfg0):
    s = cfg0["vsrc"]
    t = O.transform(s, S.rigid(np.eye(3), (5.0, 0, 0)).astype(np.float32))
    res = ctx.icp(ctx.upload(s), ctx.upload(t), ctx.icp_params(max_correspondence_distance=0.05))
    assert res.status == L.NO_CORRESPONDENCES and not res.converged
    np.testing.assert_allclose(res.transform, np.eye(4))


def test_icp_registered_cloud(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    res, reg = ctx.icp(ctx.upload(s), ctx.upload(t), ctx.icp_params(max_correspondence_distance=0.05),
                       want_registered=True)
    _cmp_points(reg.download(), O.transform(s, res.transform))


def test_icp_guess_and_max_iterations(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=3, euclidean_fitness_epsilon=1e-14)
    guess = cfg0["pair"].T_gt.astype(np.float32)
    g = ctx.icp(ctx.upload(s), ctx.upload(t), prm, guess=guess)
    o = O.icp(s, t, max_corr_dist=0.05, max_iterations=3, euclidean_fitness_epsilon=1e-14, guess=guess)
    assert g.iterations == o["iterations"] == 3 and g.state == o["state"] == 1 and g.converged
    _assert_transform_close(g.transform64, o["transform"], _extent(s), at=_centroid(s))


def test_icp_invalid_iterations(ctx, cfg0):
    c = ctx.upload(cfg0["vsrc"])
    with pytest.raises(L.LcrError) as e:
        ctx.icp(c, c, ctx.icp_params(max_iterations=0))
    assert e.value.status == L.INVALID_ARG


# -------------------------------------------------------- accumulate / crop
@pytest.mark.parametrize("radius", [0.0005, 0.002, 0.05])
def test_crop_redundant_bit_exact(ctx, cfg0, radius):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    g = ctx.crop_redundant(ctx.upload(s), ctx.upload(t), radius)
    o = O.crop_redundant(s, t, radius)
    np.testing.assert_array_equal(g.astype(bool), o)


def test_accumulate_matches_oracle(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    out, rem = ctx.accumulate(ctx.upload(s), ctx.upload(t), radius=0.001, k=50, std_mul=1.0)
    keep = ~O.crop_redundant(s, t, 0.001)
    r0 = s[keep]
    _, k2, _ = O.sor(r0, 50, 1.0)
    want = np.concatenate([t, r0[k2]])
    _cmp_points(out.download(), want)
    _cmp_points(rem.download(), r0[k2])


def test_accumulate_all(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    out, _ = ctx.accumulate(ctx.upload(s), ctx.upload(t), all_points=True)
    _cmp_points(out.download(), np.concatenate([t, s]))


# ------------------------------------------------- transforms / centroid
def test_transform_bit_exact(ctx, cfg0):
    s = cfg0["vsrc"]
    m = S.turntable(33.0, S.OBJECT_AXIS, (0.1, 0.2, -0.3)).astype(np.float32)
    m[:3, :3] *= 0.01  # the scale tool's matrix shape too
    _cmp_points(ctx.transform(ctx.upload(s), m).download(), O.transform(s, m))


def test_centroid(ctx, cfg0):
    s = cfg0["vsrc"]
    c = ctx.centroid(ctx.upload(s))
    np.testing.assert_allclose(c[:3], xyz_of(s).astype(np.float64).mean(0), rtol=0, atol=1e-6)
    np.testing.assert_allclose(c[:3], O.centroid(s)[:3], rtol=1e-4, atol=1e-5)


def test_empty_cloud_errors(ctx):
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    e = ctx.upload(points_from_xyz(np.zeros((0, 3))))
    assert len(e) == 0
    with pytest.raises(L.LcrError) as ex:
        ctx.icp(e, e, ctx.icp_params())
    assert ex.value.status == L.EMPTY
    assert len(ctx.voxel_grid(e, 0.01).download()) == 0


# ------------------------------------------------------------- autotuning
@pytest.mark.gpu
def test_launch_shapes_do_not_change_results(ctx, cfg0, tmp_path):
    """SOR distances, normals and ICP are bit-identical under every launch
    shape the autotuner can pick; the tuning cache round-trips."""
    from lowcost3dreconstruction_gb300.core import normals_of
    v, t = ctx.upload(cfg0["vsrc"]), ctx.upload(cfg0["vtgt"])
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=30, transformation_epsilon=1e-8)
    base = ctx.tune_get()
    outs = []
    for shape in ((2, 2, 2), (8, 8, 8), (3, 6, 1), (5, 5, 4)):
        ctx.tune_set(*shape)
        d, _ = ctx.sor_distances(v, 50)
        n = normals_of(ctx.normals(v, 30).download())
        r = ctx.icp_batch([v], [t], prm)[0]
        outs.append((d.view(np.uint32), n.view(np.uint32), r.transform64, r.iterations))
    for o in outs[1:]:
        np.testing.assert_array_equal(o[0], outs[0][0])
        np.testing.assert_array_equal(o[1], outs[0][1])
        np.testing.assert_array_equal(o[2], outs[0][2])
        assert o[3] == outs[0][3]
    cache = tmp_path / "tune.jsonl"
    first = ctx.autotune(v, t, str(cache))
    assert not first["from_cache"] and set(first["sor_ms"]) == {2, 3, 4, 5, 6, 8}
    again = ctx.autotune(v, t, str(cache))
    assert again["from_cache"]
    assert [again[k] for k in ("sor_warps", "normals_warps", "icp_blocks_per_sm")] == \
        [first[k] for k in ("sor_warps", "normals_warps", "icp_blocks_per_sm")]
    ctx.tune_set(base["sor_warps"], base["normals_warps"], base["icp_blocks_per_sm"])


# ------------------------------------------- isolated points (escaped lanes)
def _with_fragments(pts, seed):
    """Small fragments (3 points, 2 mm apart) far from the cloud: their k-th
    neighbour lies beyond the histogram range their tile gives them, so their
    lanes leave the tile and are searched again on their own."""
    rng = np.random.default_rng(seed)
    c = xyz_of(pts).astype(np.float64).mean(0)
    frags = []
    for j in range(6):
        d = rng.normal(size=3)
        base = c + 0.4 * d / np.linalg.norm(d)
        frags.append(base + np.array([[0, 0, 0], [0.002, 0, 0], [0, 0.002, 0]]))
    extra = random_cloud(18, seed)
    f = np.concatenate(frags).astype(np.float32)
    extra["x"], extra["y"], extra["z"] = f[:, 0], f[:, 1], f[:, 2]
    return np.concatenate([pts, extra])


def test_isolated_fragments_sor_bit_exact(ctx, cfg0):
    pts = _with_fragments(cfg0["vsrc"], 41)
    gd, _ = ctx.sor_distances(ctx.upload(pts), 50)
    od, _, _ = O.sor(pts, 50, 1.0)
    np.testing.assert_array_equal(gd.view(np.uint32), od.view(np.uint32))


@pytest.mark.parametrize("k", [30, 50])
def test_isolated_fragments_normals(ctx, cfg0, k):
    pts = _with_fragments(cfg0["vsrc"], 42)
    g = ctx.normals(ctx.upload(pts), k).download()
    o = O.normals(pts, k)
    ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
    ok = o["curvature"] < 0.2
    ang = np.arccos(np.clip(np.abs(np.sum(ng * no, axis=1)[ok]), -1, 1))
    assert np.percentile(ang, 99.9) < 1e-3
    # the fragments' own neighbourhoods (two near points, the rest ~0.4 m off)
    fr = slice(len(pts) - 18, len(pts))
    ang_fr = np.arccos(np.clip(np.abs(np.sum(ng[fr] * no[fr], axis=1)), -1, 1))
    assert np.all(ang_fr < 1e-2), ang_fr
    np.testing.assert_allclose(g["curvature"][fr], o["curvature"][fr], atol=1e-3)
