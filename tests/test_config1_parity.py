"""Parity of the exact pipeline the headline pair bench times (one config-1
pair: two 10-frame 640x480 uint16 bursts, ZE-mean, back-projection in metres,
VoxelGrid 1 mm, StatisticalOutlierRemoval k=50 mul 1.0, NormalEstimation k=30
of the inliers from SOR's neighbour lists, point-to-plane ICP with the bench's
parameters), stage by stage against the CPU oracle run on the same inputs.

Bars (the benchmark spec's): back-projection and the VoxelGrid output (where a
capture's extent overflows the voxel index, PCL's rule returns the input)
bit-exact; SOR distances,
statistics and masks bit-exact; normals within 1e-3 rad at the
99.9th percentile and curvature within 1e-4 of the FP64 oracle; the final ICP
transform within 1e-5 rad and 1e-6 x cloud extent, iteration counts within 1.
References: outlier_removal.cpp:80-84, normal_estimation.cpp:84-118,
fine_registration.cpp:105-127.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import bench as B
from lowcost3dreconstruction_gb300 import _lib as L
from lowcost3dreconstruction_gb300 import synthetic as S
from lowcost3dreconstruction_gb300.core import normals_of, xyz_of
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _bits_equal(a, b, fields):
    assert len(a) == len(b)
    for f in fields:
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32), err_msg=f)
        else:
            np.testing.assert_array_equal(x, y, err_msg=f)


ALL = ("x", "y", "z", "normal_x", "normal_y", "normal_z", "curvature", "r", "g", "b")


def _rot_angle(Ta, Tb) -> float:
    R = np.asarray(Ta, np.float64)[:3, :3] @ np.asarray(Tb, np.float64)[:3, :3].T
    return float(np.arccos(np.clip((np.trace(R) - 1) / 2, -1, 1)))


def _trans_at(Ta, Tb, at) -> float:
    p = np.r_[np.asarray(at, np.float64), 1.0]
    return float(np.linalg.norm((np.asarray(Ta, np.float64) - np.asarray(Tb, np.float64)) @ p))


@pytest.fixture(scope="module")
def c1(ctx):
    """Both captures of the bench's pair through every stage, GPU and oracle."""
    O.set_threads(os.cpu_count() or 1)
    pr = B.make_inputs(1)
    p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=10, scale=0.001, depth_max=4000.0, normals=False)
    op = O.bp_params(640, 480, scale=0.001, depth_max=4000.0, normals=False)
    out = dict(pair=pr, gpu=[], orc=[])
    for frames in (pr.src_frames, pr.tgt_frames):
        bp = ctx.backproject(frames, p)
        vg = ctx.voxel_grid(bp, 0.001)
        inl, outl, st = ctx.sor(vg, 50, 1.0, want_outliers=True)
        d, _ = ctx.sor_distances(vg, 50)
        nrm = ctx.normals(inl, 30)
        out["gpu"].append(dict(bp=bp.download(), vg=vg.download(), inl=inl.download(), outl=outl.download(),
                               st=st, d=d, nrm_cloud=nrm, nrm=nrm.download()))
        obp = O.backproject_v1(O.ze_mean_u16(frames), op)
        ovg, ov = O.voxel_grid(obp, 0.001)
        od, okeep, ost = O.sor(ovg, 50, 1.0)
        out["orc"].append(dict(bp=obp, vg=ovg, overflow=ov, d=od, keep=okeep, st=ost,
                               nrm=O.normals(ovg[okeep], 30)))
    return out


def test_config1_backprojection_and_voxels_bit_exact(c1):
    """A capture spans metres (the background), and its 1 mm voxel index range
    sits close to int32's limit: where it exceeds it, PCL's VoxelGrid warns and
    returns its input, and so do the oracle and the GPU (one of the two
    captures, depending on the last float bits of the synthetic scene; at ~2 mm
    pixel spacing every point of the other keeps a voxel of its own).  Both
    sides agree point for point either way."""
    for g, o in zip(c1["gpu"], c1["orc"]):
        _bits_equal(g["bp"], o["bp"], ALL)
        assert len(g["bp"]) > 250_000
        _bits_equal(g["vg"], o["vg"], ALL)
        if o["overflow"]:
            _bits_equal(g["vg"], g["bp"], ALL)


def test_config1_sor_bit_exact(c1):
    for g, o in zip(c1["gpu"], c1["orc"]):
        np.testing.assert_array_equal(g["d"].view(np.uint32), o["d"].view(np.uint32))
        st, ost = g["st"], o["st"]
        assert (st.mean, st.stddev, st.threshold) == (ost["mean"], ost["stddev"], ost["threshold"])
        assert st.kept == int(o["keep"].sum()) and st.removed == int((~o["keep"]).sum())
        _bits_equal(g["inl"], o["vg"][o["keep"]], ALL)
        _bits_equal(g["outl"], o["vg"][~o["keep"]], ALL)


def test_config1_sor_mask_equals_sequential_order(c1):
    """PCL sums the mean distances sequentially; the GPU uses a fixed blocked
    order.  The two thresholds differ in the last bits only, and no point lies
    that close to the threshold, so the masks are identical."""
    for g, o in zip(c1["gpu"], c1["orc"]):
        _, seq_keep, seq = O.sor(o["vg"], 50, 1.0, sequential=True)
        thr_gap = abs(seq["threshold"] - g["st"].threshold)
        assert thr_gap <= 1e-12 * seq["threshold"], thr_gap
        margin = np.min(np.abs(o["d"].astype(np.float64) - seq["threshold"]))
        assert margin > thr_gap
        np.testing.assert_array_equal(seq_keep, o["keep"])


def test_config1_normals_from_sor_lists(c1):
    for g, o in zip(c1["gpu"], c1["orc"]):
        _bits_equal(g["nrm"], o["nrm"], ("x", "y", "z", "r", "g", "b"))
        ng, no = normals_of(g["nrm"]).astype(np.float64), normals_of(o["nrm"]).astype(np.float64)
        dot = np.sum(ng * no, axis=1)
        ok = o["nrm"]["curvature"] < 0.2
        ang = np.arccos(np.clip(np.abs(dot[ok]), -1, 1))
        assert np.percentile(ang, 99.9) < 1e-3, np.percentile(ang, 99.9)
        assert np.mean(dot[ok] > 0) > 0.999
        np.testing.assert_allclose(g["nrm"]["curvature"][ok], o["nrm"]["curvature"][ok], atol=1e-4)


def _icp_oracle(src, tgt):
    P = B.ICP
    return O.icp(src, tgt, max_corr_dist=P["max_correspondence_distance"], max_iterations=P["max_iterations"],
                 transformation_epsilon=P["transformation_epsilon"],
                 euclidean_fitness_epsilon=P["euclidean_fitness_epsilon"], point_to_plane=True)


def test_config1_icp_same_inputs(ctx, c1):
    """ICP alone: the GPU's preprocessed clouds into both implementations."""
    gs, gt = c1["gpu"]
    res = ctx.icp(gs["nrm_cloud"], gt["nrm_cloud"], ctx.icp_params(**B.ICP))
    o = _icp_oracle(gs["nrm"], gt["nrm"])
    xs = xyz_of(gs["nrm"]).astype(np.float64)
    ext = float(np.max(xs.max(0) - xs.min(0)))
    assert res.converged and o["converged"]
    assert abs(res.iterations - o["iterations"]) <= 1, (res.iterations, o["iterations"])
    assert _rot_angle(res.transform64, o["transform"]) <= 1e-5
    assert _trans_at(res.transform64, o["transform"], xs.mean(0)) <= 1e-6 * ext
    assert S.rmse(res.transform64, c1["pair"].T_gt, xs) <= B.RMSE_LIMIT


def test_config1_icp_end_to_end(ctx, c1):
    """The whole pipeline on each side (the oracle from its own normals): the
    transform the bench reports against the oracle's."""
    gs, gt = c1["gpu"]
    res = ctx.icp(gs["nrm_cloud"], gt["nrm_cloud"], ctx.icp_params(**B.ICP))
    os_, ot = c1["orc"]
    o = _icp_oracle(os_["nrm"], ot["nrm"])
    xs = xyz_of(os_["nrm"]).astype(np.float64)
    ext = float(np.max(xs.max(0) - xs.min(0)))
    assert res.converged and o["converged"]
    assert abs(res.iterations - o["iterations"]) <= 1, (res.iterations, o["iterations"])
    assert _rot_angle(res.transform64, o["transform"]) <= 1e-5
    assert _trans_at(res.transform64, o["transform"], xs.mean(0)) <= 1e-6 * ext
    assert S.rmse(o["transform"], c1["pair"].T_gt, xs) <= B.RMSE_LIMIT
