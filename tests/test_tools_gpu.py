"""The remaining tool paths end to end on the GPU against the oracle:
centroid_align (centroid_align.cpp:102-130) through the C ABI and the tool,
normal_estimation's viewpoint and flip options (normal_estimation.cpp:98-118),
accumulate_clouds --negative (accumulate_clouds.cpp:130-134), CropBox on
non-finite points (accumulate_clouds.cpp:100-111) and scale (scale.cpp:68-70).
The CPU tests at the bottom pin the oracle's own CropBox semantics."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import random_cloud
from lowcost3dreconstruction_gb300.core import normals_of, xyz_of
from oracle import oracle as O

ROOT = Path(__file__).resolve().parents[1]
BIN = ROOT / "lowcost3dreconstruction_gb300" / "bin"


def run(tool, *args):
    return subprocess.run([str(BIN / tool), *map(str, args)], capture_output=True, text=True, timeout=120)


@pytest.fixture(scope="module")
def tools():
    from lowcost3dreconstruction_gb300 import build
    build.build_lib()
    build.build_tools()


def _bits(a, b, fields=("x", "y", "z", "normal_x", "normal_y", "normal_z", "curvature", "r", "g", "b")):
    assert len(a) == len(b)
    for f in fields:
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32), err_msg=f)
        else:
            np.testing.assert_array_equal(x, y, err_msg=f)


# ------------------------------------------------------------ centroid_align
ANGLES = [(0.0, 0.0, 0.0, 0.0), (10.0, -20.0, 35.0, 0.05), (-90.0, 45.0, 180.0, -0.2)]


@pytest.mark.gpu
@pytest.mark.parametrize("roll,pitch,yaw,elev", ANGLES)
def test_centroid_align_chain(ctx, cfg0, roll, pitch, yaw, elev):
    """T = Tr(0, e, 0) Tr(c_t) Rx(roll) Ry(pitch) Rz(yaw) Tr(-c_s), points and
    normals moved.  Against the FP64 chain the GPU (FP64 centroids, one float
    matrix) agrees to FP32 rounding; against PCL's float chain (sequential FP32
    centroids, four passes) to that chain's own centroid error."""
    s = O.normals(cfg0["vsrc"], 30)
    t = cfg0["vtgt"]
    out, m = ctx.centroid_align(ctx.upload(s), ctx.upload(t), roll, pitch, yaw, elev)
    g = out.download()
    want, M = O.centroid_align(s, t, roll, pitch, yaw, elev, exact=True)
    np.testing.assert_allclose(m.astype(np.float64), M, rtol=0, atol=2e-7)
    np.testing.assert_allclose(xyz_of(g), xyz_of(want), rtol=0, atol=1e-6)
    np.testing.assert_allclose(normals_of(g), normals_of(want), rtol=0, atol=1e-6)
    pcl, _ = O.centroid_align(s, t, roll, pitch, yaw, elev, exact=False)
    cerr = max(np.abs(O.centroid(s)[:3] - xyz_of(s).astype(np.float64).mean(0)).max(),
               np.abs(O.centroid(t)[:3] - xyz_of(t).astype(np.float64).mean(0)).max())
    assert np.abs(xyz_of(g).astype(np.float64) - xyz_of(pcl)).max() <= 2 * cerr + 4e-6
    # the moved source's centroid sits on the target's, lifted by the elevation
    c = xyz_of(g).astype(np.float64).mean(0)
    np.testing.assert_allclose(c, xyz_of(t).astype(np.float64).mean(0) + [0.0, elev, 0.0], atol=2e-6)


@pytest.mark.gpu
def test_centroid_align_tool(tmp_path, tools, cfg0):
    from lowcost3dreconstruction_gb300 import _lib as L
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    L.write_ply(tmp_path / "s.ply", s)
    L.write_ply(tmp_path / "t.ply", t)
    r = run("centroid_align", "-i", tmp_path / "s.ply", "-t", tmp_path / "t.ply", "-o", tmp_path / "o.ply",
            "-a", tmp_path / "acc.ply", "-r", "10", "-p", "-20", "-y", "35", "-e", "0.05")
    assert r.returncode == 0, r.stderr
    want, _ = O.centroid_align(s, t, 10.0, -20.0, 35.0, 0.05, exact=True)
    got = L.read_ply(tmp_path / "o.ply")
    np.testing.assert_allclose(xyz_of(got), xyz_of(want), rtol=0, atol=1e-6)
    acc = L.read_ply(tmp_path / "acc.ply")
    assert len(acc) == len(s) + len(t)
    np.testing.assert_array_equal(acc["x"][:len(s)], got["x"])


# ------------------------------------------------------ normal_estimation flags
@pytest.mark.gpu
@pytest.mark.parametrize("flags", [[], ["-r"], ["-c"], ["-c", "-r"], ["-z"], ["-z", "-r"]])
def test_normal_estimation_viewpoint_options(tmp_path, tools, cfg0, flags):
    """-c: the centroid is the viewpoint, then every normal is negated (outwards)
    unless -r; -z: the sensor origin (0, 0, 0 for a PLY without one); -r alone
    negates the origin-facing normals."""
    from lowcost3dreconstruction_gb300 import _lib as L
    pts = cfg0["vsrc"]
    L.write_ply(tmp_path / "in.ply", pts)
    r = run("normal_estimation", "-i", tmp_path / "in.ply", "-o", tmp_path / "out.ply", "-n", "30", *flags)
    assert r.returncode == 0, r.stderr
    g = L.read_ply(tmp_path / "out.ply")
    centroid, reverse = "-c" in flags, "-r" in flags
    vp = O.centroid(pts)[:3] if centroid else (0.0, 0.0, 0.0)
    o = O.normals(pts, 30, viewpoint=vp, flip_all=(centroid and not reverse) or (not centroid and reverse))
    _bits(g, o, ("x", "y", "z", "r", "g", "b"))
    ng, no = normals_of(g).astype(np.float64), normals_of(o).astype(np.float64)
    dot = np.sum(ng * no, axis=1)
    ok = o["curvature"] < 0.2
    assert np.percentile(np.arccos(np.clip(np.abs(dot[ok]), -1, 1)), 99.9) < 1e-3
    assert np.mean(dot[ok] > 0) > 0.999   # the same orientation, not just the same line


@pytest.mark.gpu
def test_normal_estimation_rejects_centroid_with_origin(tmp_path, tools, cfg0):
    from lowcost3dreconstruction_gb300 import _lib as L
    L.write_ply(tmp_path / "in.ply", cfg0["vsrc"][:100])
    r = run("normal_estimation", "-i", tmp_path / "in.ply", "-o", tmp_path / "o.ply", "-c", "-z")
    assert r.returncode == 255 and "at the same time" in r.stderr


# ----------------------------------------------------- accumulate --negative
@pytest.mark.gpu
def test_accumulate_negative_writes_the_remaining_points(tmp_path, tools, cfg0):
    from lowcost3dreconstruction_gb300 import _lib as L
    s, t = cfg0["vsrc"], cfg0["vtgt"]
    L.write_ply(tmp_path / "s.ply", s)
    L.write_ply(tmp_path / "t.ply", t)
    r = run("accumulate_clouds", "-i", tmp_path / "s.ply", "-t", tmp_path / "t.ply", "-o", tmp_path / "acc.ply",
            "-r", "0.001", "-c", "50", "-d", "1.0", "-n")
    assert r.returncode == 0, r.stderr
    keep = ~O.crop_redundant(s, t, 0.001)
    r0 = s[keep]
    _, k2, _ = O.sor(r0, 50, 1.0)
    _bits(L.read_ply(tmp_path / "acc_negative.ply"), r0[k2])
    _bits(L.read_ply(tmp_path / "acc.ply"), np.concatenate([t, r0[k2]]))


# ------------------------------------------------------- CropBox, non-finite
def _with_nonfinite(pts, every=37):
    p = pts.copy()
    p["x"][::every] = np.nan
    p["z"][5::every] = np.inf
    return p


@pytest.mark.gpu
def test_crop_drops_nonfinite_source_points(ctx, cfg0):
    s, t = _with_nonfinite(cfg0["vsrc"]), cfg0["vtgt"]
    g = ctx.crop_redundant(ctx.upload(s), ctx.upload(t), 0.002).astype(bool)
    o = O.crop_redundant(s, t, 0.002)
    np.testing.assert_array_equal(g, o)
    bad = ~(np.isfinite(s["x"]) & np.isfinite(s["y"]) & np.isfinite(s["z"]))
    assert np.all(g[bad])


@pytest.mark.gpu
def test_crop_with_a_nonfinite_target_point_removes_everything(ctx, cfg0):
    s, t = cfg0["vsrc"], cfg0["vtgt"].copy()
    t["y"][1000] = np.nan
    g = ctx.crop_redundant(ctx.upload(s), ctx.upload(t), 0.002).astype(bool)
    assert np.all(g) and np.all(O.crop_redundant(s, t, 0.002))
    # and an empty target removes nothing, non-finite source points included
    e = ctx.upload(t[:0])
    sn = _with_nonfinite(s)
    assert not ctx.crop_redundant(ctx.upload(sn), e, 0.002).any()
    assert not O.crop_redundant(sn, t[:0], 0.002).any()


# ------------------------------------------------------------------- scale
@pytest.mark.gpu
@pytest.mark.parametrize("factor", ["0.001", "10", "2.5"])
def test_scale_tool_bit_exact(tmp_path, tools, cfg0, factor):
    from lowcost3dreconstruction_gb300 import _lib as L
    pts = O.normals(cfg0["vsrc"], 30)
    L.write_ply(tmp_path / "in.ply", pts)
    r = run("scale", "-i", tmp_path / "in.ply", "-o", tmp_path / "out.ply", "-s", factor)
    assert r.returncode == 0, r.stderr
    m = np.eye(4, dtype=np.float32)
    m[0, 0] = m[1, 1] = m[2, 2] = np.float32(float(factor))
    _bits(L.read_ply(tmp_path / "out.ply"), O.transform(pts, m))


# --------------------------------------------------------------------- CPU
def test_oracle_crop_nonfinite_semantics():
    s = random_cloud(400, 3, scale=0.05)
    t = random_cloud(300, 4, scale=0.05)
    base = O.crop_redundant(s, t, 0.004)
    sn = _with_nonfinite(s, 11)
    got = O.crop_redundant(sn, t, 0.004)
    bad = ~(np.isfinite(sn["x"]) & np.isfinite(sn["z"]))
    assert np.all(got[bad]) and np.array_equal(got[~bad], base[~bad])
    tn = t.copy()
    tn["z"][7] = np.nan
    assert np.all(O.crop_redundant(s, tn, 0.004))
    assert not O.crop_redundant(sn, t[:0], 0.004).any()


def test_oracle_centroid_align_chain_forms_agree():
    s = random_cloud(2000, 5, scale=0.2)
    t = random_cloud(1500, 6, scale=0.2)
    a, M = O.centroid_align(s, t, 10.0, -20.0, 35.0, 0.05, exact=True)
    b, M2 = O.centroid_align(s, t, 10.0, -20.0, 35.0, 0.05, exact=False)
    np.testing.assert_allclose(M, M2, atol=1e-6)
    np.testing.assert_allclose(xyz_of(a), xyz_of(b), atol=1e-5)
    # the rotation block is Rx Ry Rz in that order
    r, p, y = np.deg2rad([10.0, -20.0, 35.0])
    Rx = np.array([[1, 0, 0], [0, np.cos(r), -np.sin(r)], [0, np.sin(r), np.cos(r)]])
    Ry = np.array([[np.cos(p), 0, np.sin(p)], [0, 1, 0], [-np.sin(p), 0, np.cos(p)]])
    Rz = np.array([[np.cos(y), -np.sin(y), 0], [np.sin(y), np.cos(y), 0], [0, 0, 1]])
    np.testing.assert_allclose(M[:3, :3], Rx @ Ry @ Rz, atol=1e-15)
