"""Generates the golden fixtures in this folder from the CPU oracle on small
seeded inputs.  The fixtures pin the oracle's own outputs (a regression guard
for the oracle); the reference itself has no tests or vectors to pin to.

    python tests/golden/make_golden.py            # every fixture
    python tests/golden/make_golden.py sr sfm     # only the named fixtures (sr, sfm, posenet)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))

from lowcost3dreconstruction_gb300 import build  # noqa: E402
from lowcost3dreconstruction_gb300.core import points_from_xyz, xyz_of, normals_of  # noqa: E402


def cloud(rng, n, scale=0.1, lattice=0.0):
    xyz = rng.uniform(-scale, scale, (n, 3)).astype(np.float32)
    if lattice:
        xyz = (np.round(xyz / lattice) * lattice).astype(np.float32)
    return xyz


def main() -> None:
    build.build_oracle()
    from oracle import oracle as O
    rng = np.random.default_rng(20260101)
    g = {}
    # kNN with ties (lattice) and duplicates
    ref = cloud(rng, 400, lattice=0.02)
    ref[::17] = ref[1::17][: len(ref[::17])]
    qry = cloud(rng, 100, lattice=0.02)
    g["knn_ref"], g["knn_qry"] = ref, qry
    g["knn_idx"], g["knn_dist"] = O.knn(points_from_xyz(ref), points_from_xyz(qry), 8)
    # voxel grid (means of xyz, normals, colour)
    vx = cloud(rng, 2000, scale=0.05)
    vn = rng.normal(size=(2000, 3)).astype(np.float32)
    vc = rng.integers(0, 256, (2000, 3)).astype(np.uint8)
    g["vox_xyz"], g["vox_nrm"], g["vox_rgb"] = vx, vn, vc
    out, _ = O.voxel_grid(points_from_xyz(vx, vn, vc), 0.01)
    g["vox_out_xyz"], g["vox_out_nrm"] = xyz_of(out), normals_of(out)
    g["vox_out_rgb"] = np.stack([out["r"], out["g"], out["b"]], 1)
    # SOR
    sx = cloud(rng, 800, scale=0.05)
    sx[5] = (0.5, 0.5, 0.5)
    g["sor_xyz"] = sx
    d, keep, st = O.sor(points_from_xyz(sx), 10, 1.0)
    g["sor_dist"], g["sor_keep"] = d, keep
    g["sor_stats"] = np.array([st["mean"], st["stddev"], st["threshold"]])
    # normals on a bumpy surface
    uv = rng.uniform(-0.05, 0.05, (800, 2))
    nx = np.c_[uv, 0.05 * np.sin(40 * uv[:, 0]) - 1.0].astype(np.float32)
    g["ne_xyz"] = nx
    ne = O.normals(points_from_xyz(nx), 12)
    g["ne_nrm"], g["ne_curv"] = normals_of(ne), ne["curvature"]
    # point-to-point ICP
    ix = rng.uniform(-0.1, 0.1, (1500, 3))
    ix[:, 2] += 0.2 * np.sin(9 * ix[:, 0]) * np.cos(7 * ix[:, 1])
    a = np.deg2rad(4.0)
    R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
    tx = ix @ R.T + np.array([0.005, 0.0, -0.003])
    g["icp_src"], g["icp_tgt"] = ix.astype(np.float32), tx.astype(np.float32)
    r = O.icp(points_from_xyz(ix), points_from_xyz(tx), max_corr_dist=0.05, max_iterations=30,
              transformation_epsilon=1e-10)
    g["icp_T"], g["icp_iters"] = r["transform"], np.array(r["iterations"])
    # depth: burst ZE-mean and Kinect v1 back-projection with image normals
    fr = rng.integers(900, 1100, (5, 24, 32)).astype(np.uint16)
    fr[rng.random(fr.shape) < 0.3] = 0
    g["ze_frames"] = fr
    fused = O.ze_mean_u16(fr)
    g["ze_fused"] = fused
    bp = O.backproject_v1(fused, O.bp_params(32, 24, fx=30.0, fy=30.0, cx=15.5, cy=11.5, scale=0.001,
                                             depth_min=950, normals=True))
    g["bp_xyz"], g["bp_nrm"] = xyz_of(bp), normals_of(bp)
    np.savez_compressed(HERE / "oracle_small.npz", **g)
    print("wrote", HERE / "oracle_small.npz", sum(v.nbytes for v in g.values()), "bytes raw")


def sr_fixtures() -> None:
    """The super-resolution oracle (oracle/sr.py) on a 4-frame 40 x 48 burst of
    a smooth scene under small rigid motions with 1% holes, uint16 and float."""
    from oracle import sr as OS
    rng = np.random.default_rng(20261204)
    h, w = 40, 48
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    frames = []
    for f in range(4):
        a = 0.0 if f == 0 else np.deg2rad(rng.uniform(-0.4, 0.4))
        tx, ty = (0.0, 0.0) if f == 0 else rng.uniform(-0.6, 0.6, 2)
        X = np.cos(a) * x - np.sin(a) * y + tx
        Y = np.sin(a) * x + np.cos(a) * y + ty
        d = 1000 + 90 * np.sin(X / 6.0) * np.cos(Y / 5.0) + 0.5 * X + rng.normal(0, 0.3, x.shape)
        d[rng.random(d.shape) < 0.01] = 0
        frames.append(np.clip(np.rint(d), 0, 65535).astype(np.uint16))
    frames = np.stack(frames)
    g = {"frames": frames}
    g["fused"], g["warps"], g["iters"] = OS.super_resolve(frames, 4, 30, 1e-10)
    ff = frames.astype(np.float32) + rng.uniform(-0.5, 0.5, frames.shape).astype(np.float32)
    ff[frames == 0] = 0
    g["frames_f32"] = ff
    g["fused_f32"], g["warps_f32"], g["iters_f32"] = OS.super_resolve(ff, 4, 30, 1e-10)
    np.savez_compressed(HERE / "sr_small.npz", **g)
    print("wrote", HERE / "sr_small.npz", sum(v.nbytes for v in g.values()), "bytes raw")


def sfm_fixtures() -> None:
    """The SfM filters' oracle (oracle/sfm.py) on a 3000-point floor with two
    blobs, stray points and NaN records: the CropBox masks, the Euclidean
    cluster labels and the RANSAC plane with its inliers and hypothesis counts."""
    from oracle import sfm as OF
    rng = np.random.default_rng(20261205)
    floor = np.c_[rng.uniform(-0.5, 0.5, (2400, 2)), rng.normal(0, 0.002, 2400)]
    blobs = [rng.normal(c, 0.02, (m, 3)) for c, m in (((0.2, 0.1, 0.2), 300), ((-0.2, -0.1, 0.25), 200))]
    xyz = np.concatenate([floor] + blobs + [rng.uniform(-0.5, 0.5, (100, 3))]).astype(np.float32)
    xyz = xyz[rng.permutation(len(xyz))]
    xyz[::97] = np.nan
    g = {"xyz": xyz}
    g["crop_in"], g["crop_out"] = OF.crop_box(xyz, (-0.25, -0.25, -0.05), (0.25, 0.25, 0.3))
    g["labels"], nk = OF.euclidean_clusters(xyz, 0.03, 50, len(xyz))
    g["nclusters"] = np.array(nk)
    c, inl, counts, best = OF.plane_segment(xyz, 0.01, 64, 7)
    g["plane"], g["plane_inliers"], g["plane_counts"], g["plane_best"] = c, inl, counts, np.array(best)
    np.savez_compressed(HERE / "sfm_small.npz", **g)
    print("wrote", HERE / "sfm_small.npz", sum(v.nbytes for v in g.values()), "bytes raw")


def posenet_fixtures() -> None:
    """The pose network's oracle forward (oracle/posenet.py) on seeded weights
    (scaled normal draws of the seed below) and two pairs of 1024-point clouds:
    features, max-pool winners and the head's outputs."""
    from oracle import posenet as OP
    rng = np.random.default_rng(20261206)
    params = (rng.standard_normal(OP.PARAMS) * 0.05).astype(np.float32)
    pts = rng.uniform(-0.1, 0.1, (4, 1024, 4)).astype(np.float32)
    feat, argmax, y, _ = OP.forward(params, pts)
    g = {"seed": np.array(20261206), "pts": pts, "feat": feat.astype(np.float32), "argmax": argmax.astype(np.int32),
         "y": y}
    np.savez_compressed(HERE / "posenet_small.npz", **g)
    print("wrote", HERE / "posenet_small.npz", sum(v.nbytes for v in g.values()), "bytes raw")


if __name__ == "__main__":
    only = set(sys.argv[1:])
    if not only:
        main()
    if not only or "sr" in only:
        sr_fixtures()
    if not only or "sfm" in only:
        sfm_fixtures()
    if not only or "posenet" in only:
        posenet_fixtures()
