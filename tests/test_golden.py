"""Committed fixtures (tests/golden/oracle_small.npz, made by
tests/golden/make_golden.py): the oracle must reproduce them exactly (CPU),
and the GPU path must match them at the parity bar of each stage (GPU)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

from lowcost3dreconstruction_gb300.core import points_from_xyz, xyz_of, normals_of
from oracle import oracle as O

G = np.load(Path(__file__).resolve().parent / "golden" / "oracle_small.npz")


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def _vox_in():
    return points_from_xyz(G["vox_xyz"], G["vox_nrm"], G["vox_rgb"])


def _bp_params(make):
    return make(32, 24, fx=30.0, fy=30.0, cx=15.5, cy=11.5, scale=0.001, depth_min=950, normals=True)


# ------------------------------------------------------------ oracle, CPU
def test_oracle_reproduces_knn_and_voxel_fixtures():
    idx, dist = O.knn(points_from_xyz(G["knn_ref"]), points_from_xyz(G["knn_qry"]), 8)
    np.testing.assert_array_equal(idx, G["knn_idx"])
    np.testing.assert_array_equal(_bits(dist), _bits(G["knn_dist"]))
    out, _ = O.voxel_grid(_vox_in(), 0.01)
    np.testing.assert_array_equal(_bits(xyz_of(out)), _bits(G["vox_out_xyz"]))
    np.testing.assert_array_equal(_bits(normals_of(out)), _bits(G["vox_out_nrm"]))


def test_oracle_reproduces_sor_normals_icp_depth_fixtures():
    d, keep, st = O.sor(points_from_xyz(G["sor_xyz"]), 10, 1.0)
    np.testing.assert_array_equal(_bits(d), _bits(G["sor_dist"]))
    np.testing.assert_array_equal(keep, G["sor_keep"])
    assert [st["mean"], st["stddev"], st["threshold"]] == list(G["sor_stats"])
    ne = O.normals(points_from_xyz(G["ne_xyz"]), 12)
    np.testing.assert_array_equal(_bits(normals_of(ne)), _bits(G["ne_nrm"]))
    r = O.icp(points_from_xyz(G["icp_src"]), points_from_xyz(G["icp_tgt"]), max_corr_dist=0.05,
              max_iterations=30, transformation_epsilon=1e-10)
    np.testing.assert_array_equal(r["transform"], G["icp_T"])
    fused = O.ze_mean_u16(G["ze_frames"])
    np.testing.assert_array_equal(fused, G["ze_fused"])
    bp = O.backproject_v1(fused, _bp_params(O.bp_params))
    np.testing.assert_array_equal(_bits(xyz_of(bp)), _bits(G["bp_xyz"]))
    np.testing.assert_array_equal(_bits(normals_of(bp)), _bits(G["bp_nrm"]))


# -------------------------------------------------------------- GPU path
@pytest.mark.gpu
def test_gpu_matches_fixtures(ctx):
    from lowcost3dreconstruction_gb300 import _lib as L
    gi, gd = ctx.knn(ctx.upload(points_from_xyz(G["knn_ref"])), ctx.upload(points_from_xyz(G["knn_qry"])), 8)
    np.testing.assert_array_equal(gi, G["knn_idx"])
    np.testing.assert_array_equal(_bits(gd), _bits(G["knn_dist"]))
    v = ctx.voxel_grid(ctx.upload(_vox_in()), 0.01).download()
    np.testing.assert_array_equal(_bits(xyz_of(v)), _bits(G["vox_out_xyz"]))
    np.testing.assert_array_equal(_bits(normals_of(v)), _bits(G["vox_out_nrm"]))
    sd, st = ctx.sor_distances(ctx.upload(points_from_xyz(G["sor_xyz"])), 10)
    np.testing.assert_array_equal(_bits(sd), _bits(G["sor_dist"]))
    ne = ctx.normals(ctx.upload(points_from_xyz(G["ne_xyz"])), 12).download()
    dot = np.abs(np.sum(normals_of(ne).astype(np.float64) * G["ne_nrm"], axis=1))
    assert np.min(dot) > 1 - 1e-6
    np.testing.assert_allclose(ne["curvature"], G["ne_curv"], atol=1e-5)
    res = ctx.icp(ctx.upload(points_from_xyz(G["icp_src"])), ctx.upload(points_from_xyz(G["icp_tgt"])),
                  ctx.icp_params(max_correspondence_distance=0.05, max_iterations=30, transformation_epsilon=1e-10))
    np.testing.assert_allclose(res.transform64, G["icp_T"], atol=1e-6)
    p = ctx.depth_params(L.KINECT_V1, 32, 24, frames=5, fx=30.0, fy=30.0, cx=15.5, cy=11.5, scale=0.001,
                         depth_min=950, normals=True)
    bp = ctx.backproject(G["ze_frames"], p).download()
    np.testing.assert_array_equal(_bits(xyz_of(bp)), _bits(G["bp_xyz"]))
    np.testing.assert_array_equal(_bits(normals_of(bp)), _bits(G["bp_nrm"]))
