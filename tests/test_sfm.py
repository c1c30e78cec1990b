"""SfM-side filters: CropBox, Euclidean clusters, RANSAC plane
(pcl_tools/crop_cloud.cpp, cluster_extraction.cpp, planar_segmentation.cpp).

CPU: the oracle on hand-made cases.  GPU: the library against the oracle --
crop masks and cluster labels bit-exact (both are decided on exact FP32
quantities), the plane's hypothesis winner exact and its refitted
coefficients within FP64-summation-order tolerance; and the tools."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import sfm as O

BIN = Path(__file__).resolve().parents[1] / "lowcost3dreconstruction_gb300" / "bin"


def scene(seed=0, n_plane=20000, nan_frac=0.002):
    """A noisy floor (z ~ 0), three blobs above it, scattered points, some NaNs."""
    rng = np.random.default_rng(seed)
    floor = np.c_[rng.uniform(-1, 1, (n_plane, 2)), rng.normal(0, 0.003, n_plane)]
    blobs = [rng.normal(c, 0.04, (m, 3)) for c, m in (((0.3, 0.2, 0.4), 3000), ((-0.4, -0.1, 0.5), 2000),
                                                          ((0.0, 0.6, 0.3), 800))]
    scatter = rng.uniform(-1, 1, (300, 3)) * np.r_[1, 1, 0.5] + np.r_[0, 0, 0.6]
    xyz = np.concatenate([floor] + blobs + [scatter]).astype(np.float32)
    xyz = xyz[rng.permutation(len(xyz))]
    xyz[rng.random(len(xyz)) < nan_frac] = np.nan
    return xyz


# ------------------------------------------------------------------ CPU
def test_oracle_clusters_small_case():
    xyz = np.array([[0, 0, 0], [0.05, 0, 0], [0.2, 0, 0], [1, 1, 1], [1.05, 1, 1], [1.04, 1.04, 1], [np.nan] * 3],
                   np.float32)
    labels, k = O.euclidean_clusters(xyz, 0.1, 2, 100)
    assert k == 2
    assert list(labels) == [1, 1, -1, 0, 0, 0, -1]   # the larger cluster ranks first


def test_oracle_plane_finds_the_floor():
    xyz = scene(1)
    c, inl, counts, best = O.plane_segment(xyz, 0.01, 64, 3)
    assert abs(abs(c[2]) - 1) < 1e-3 and abs(c[3]) < 2e-3
    assert inl.sum() > 0.95 * 20000
    assert counts[best] == counts.max()


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_crop_box_matches_oracle(ctx):
    from lowcost3dreconstruction_gb300.core import points_from_xyz, xyz_of
    xyz = scene(2)
    c = ctx.upload(points_from_xyz(xyz))
    lo, hi = np.float32([-0.5, -0.25, -0.01]), np.float32([0.4, 0.7, 0.45])
    inside, outside = ctx.crop_box(c, lo, hi)
    want_in, want_out = O.crop_box(xyz, lo, hi)
    np.testing.assert_array_equal(xyz_of(inside.download()), xyz[want_in])
    np.testing.assert_array_equal(xyz_of(outside.download()), xyz[want_out])


@pytest.mark.gpu
@pytest.mark.parametrize("tol,min_size", [(0.02, 1), (0.05, 100), (0.011, 10)])
def test_euclidean_clusters_match_oracle(ctx, tol, min_size):
    from lowcost3dreconstruction_gb300.core import points_from_xyz, xyz_of
    xyz = scene(3)
    c = ctx.upload(points_from_xyz(xyz))
    labels, k, kept, rest = ctx.euclidean_clusters(c, tol, min_size, len(xyz))
    want, wk = O.euclidean_clusters(xyz, tol, min_size, len(xyz))
    assert k == wk
    np.testing.assert_array_equal(labels, want)
    order = np.concatenate([np.nonzero(want == r)[0] for r in range(wk)] or [np.zeros(0, int)])
    np.testing.assert_array_equal(xyz_of(kept.download()), xyz[order])
    np.testing.assert_array_equal(xyz_of(rest.download()), xyz[want < 0])


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [0, 7])
def test_plane_segment_matches_oracle(ctx, seed):
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    xyz = scene(4)
    c = ctx.upload(points_from_xyz(xyz))
    coef, m, plane, rest = ctx.plane_segment(c, 0.01, hypotheses=256, seed=seed)
    wc, winl, _, _ = O.plane_segment(xyz, 0.01, 256, seed)
    np.testing.assert_allclose(coef, wc, atol=2e-6)
    assert abs(m - int(winl.sum())) <= 2            # points within an ulp of the threshold
    assert len(plane) == m and len(rest) == len(xyz) - m
    assert abs(abs(coef[2]) - 1) < 1e-3


@pytest.mark.gpu
def test_sfm_tools_chain(tmp_path):
    """sfm.sh:82-85: cluster_extraction then planar_segmentation, vs the oracle."""
    from lowcost3dreconstruction_gb300 import _lib as L
    from lowcost3dreconstruction_gb300.core import points_from_xyz, xyz_of
    xyz = scene(5)
    L.write_ply(tmp_path / "m.ply", points_from_xyz(xyz))
    run = lambda *a: subprocess.run([str(BIN / a[0]), *map(str, a[1:])], capture_output=True, text=True, timeout=120)
    r = run("cluster_extraction", "-i", tmp_path / "m.ply", "-o", tmp_path / "c.ply", "--tolerance", "0.02", "-f",
            "-p", "0.1")
    assert r.returncode == 0, r.stderr
    labels, k = O.euclidean_clusters(xyz, 0.02, int(len(xyz) * 0.1), len(xyz))
    assert f"{k} cluster(s) extracted." in r.stdout
    got = xyz_of(L.read_ply(tmp_path / "c.ply"))
    np.testing.assert_array_equal(got, np.concatenate([xyz[labels == j] for j in range(k)]))
    assert len(L.read_ply(tmp_path / "c_outliers.ply")) == int((labels < 0).sum())
    r = run("planar_segmentation", "-i", tmp_path / "c.ply", "-o", tmp_path / "p.ply", "--threshold", "0.01", "-n")
    assert r.returncode == 0, r.stderr
    off, on = L.read_ply(tmp_path / "p.ply"), L.read_ply(tmp_path / "p_plane.ply")
    assert len(off) + len(on) == len(got) and len(on) > 0.9 * 20000 * 0.99
    r = run("crop_cloud", "-i", tmp_path / "m.ply", "-o", tmp_path / "x.ply", "-r", "0.3", "-n")
    assert r.returncode == 0, r.stderr
    assert len(L.read_ply(tmp_path / "x.ply")) + len(L.read_ply(tmp_path / "x_negative.ply")) == \
        int(np.all(np.isfinite(xyz), axis=1).sum())


# ------------------------------------------------------------------ fixtures
GOLD = Path(__file__).resolve().parent / "golden" / "sfm_small.npz"


def test_oracle_reproduces_the_committed_fixture():
    """tests/golden/sfm_small.npz (tests/golden/make_golden.py sfm) pins the
    oracle's own outputs: masks, labels and plane on a cloud with NaN records."""
    g = np.load(GOLD)
    xyz = g["xyz"]
    a, b = O.crop_box(xyz, (-0.25, -0.25, -0.05), (0.25, 0.25, 0.3))
    np.testing.assert_array_equal(a, g["crop_in"])
    np.testing.assert_array_equal(b, g["crop_out"])
    labels, k = O.euclidean_clusters(xyz, 0.03, 50, len(xyz))
    np.testing.assert_array_equal(labels, g["labels"])
    assert k == int(g["nclusters"])
    c, inl, counts, best = O.plane_segment(xyz, 0.01, 64, 7)
    np.testing.assert_array_equal(counts, g["plane_counts"])
    assert best == int(g["plane_best"])
    np.testing.assert_allclose(c, g["plane"], atol=1e-6)
    np.testing.assert_array_equal(inl, g["plane_inliers"])


@pytest.mark.gpu
def test_library_matches_the_committed_fixture(ctx):
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    g = np.load(GOLD)
    cloud = ctx.upload(points_from_xyz(g["xyz"]))
    labels, k, _, _ = ctx.euclidean_clusters(cloud, 0.03, 50, len(g["xyz"]))
    np.testing.assert_array_equal(labels, g["labels"])
    assert k == int(g["nclusters"])
    coef, m, _, _ = ctx.plane_segment(cloud, 0.01, 64, 7)
    np.testing.assert_allclose(coef, g["plane"], atol=2e-6)
    assert m == int(g["plane_inliers"].sum())
