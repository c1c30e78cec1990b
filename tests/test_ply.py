"""PLY I/O (host only, no GPU): round trips through the writer, and files in
the layouts the reference's tools read and write -- the capture tools' ascii
vertex list (capture/depth_capture/depth_capture.cpp:281-306: x y z nx ny nz
red green blue) and PCL's binary PointXYZRGBNormal with extra elements."""
from __future__ import annotations

import struct

import numpy as np
import pytest

from conftest import random_cloud
from lowcost3dreconstruction_gb300 import _lib as L

FIELDS = ("x", "y", "z", "normal_x", "normal_y", "normal_z", "curvature", "r", "g", "b")


@pytest.fixture(scope="module", autouse=True)
def lib():
    from lowcost3dreconstruction_gb300 import build
    build.build_lib()


@pytest.mark.parametrize("binary", [True, False])
def test_round_trip(tmp_path, binary):
    pts = random_cloud(1000, 3)
    pts["x"][7] = np.nan
    L.write_ply(tmp_path / "a.ply", pts, binary=binary)
    back = L.read_ply(tmp_path / "a.ply")
    assert len(back) == len(pts)
    for f in FIELDS:
        if pts[f].dtype.kind == "f":
            np.testing.assert_array_equal(back[f].view(np.uint32) if binary else back[f],
                                          pts[f].view(np.uint32) if binary else pts[f], err_msg=f)
        else:
            np.testing.assert_array_equal(back[f], pts[f], err_msg=f)


def test_empty_cloud_round_trip(tmp_path):
    L.write_ply(tmp_path / "e.ply", random_cloud(0, 1))
    assert len(L.read_ply(tmp_path / "e.ply")) == 0


def test_capture_tool_ascii_layout(tmp_path):
    text = ("ply\nformat ascii 1.0\nelement vertex 2\nproperty float x\nproperty float y\nproperty float z\n"
            "property float nx\nproperty float ny\nproperty float nz\nproperty uchar red\nproperty uchar green\n"
            "property uchar blue\nend_header\n"
            "-1.500000 2.250000 -1000.000000 0.0 0.0 1.0 128 128 128\n"
            "3.000000 -4.000000 -900.500000 0.6 0.0 0.8 10 20 30\n")
    (tmp_path / "c.ply").write_text(text)
    p = L.read_ply(tmp_path / "c.ply")
    np.testing.assert_array_equal(p["x"], np.float32([-1.5, 3.0]))
    np.testing.assert_array_equal(p["z"], np.float32([-1000.0, -900.5]))
    np.testing.assert_array_equal(p["normal_x"], np.float32([0.0, 0.6]))
    assert list(p["r"]) == [128, 10] and list(p["g"]) == [128, 20] and list(p["b"]) == [128, 30]


def test_binary_with_packed_rgb_and_extra_elements(tmp_path):
    hdr = ("ply\nformat binary_little_endian 1.0\ncomment PCL generated\nobj_info x\n"
           "element vertex 2\nproperty float x\nproperty float y\nproperty float z\nproperty float rgb\n"
           "property float normal_x\nproperty float normal_y\nproperty float normal_z\nproperty float curvature\n"
           "property uchar extra\n"
           "element camera 1\nproperty float view_px\nproperty float view_py\n"
           "element face 1\nproperty list uchar int vertex_indices\nend_header\n").encode()
    rgb = struct.unpack("<f", struct.pack("<I", (10 << 16) | (20 << 8) | 30))[0]
    body = b"".join(struct.pack("<8fB", x, 2 * x, 3 * x, rgb, 0.0, 1.0, 0.0, 0.25, 9) for x in (1.0, 2.0))
    body += struct.pack("<2f", 0.0, 0.0) + struct.pack("<B3i", 3, 0, 1, 1)
    (tmp_path / "b.ply").write_bytes(hdr + body)
    p = L.read_ply(tmp_path / "b.ply")
    np.testing.assert_array_equal(p["y"], np.float32([2.0, 4.0]))
    np.testing.assert_array_equal(p["curvature"], np.float32([0.25, 0.25]))
    assert list(p["r"]) == [10, 10] and list(p["g"]) == [20, 20] and list(p["b"]) == [30, 30]


def test_malformed_files_fail_cleanly(tmp_path):
    (tmp_path / "bad.ply").write_text("ply\nformat ascii 1.0\nelement vertex 2\nproperty foo x\nend_header\n")
    with pytest.raises(L.LcrError):
        L.read_ply(tmp_path / "bad.ply")
    (tmp_path / "short.ply").write_text("ply\nformat ascii 1.0\nelement vertex 3\nproperty float x\nend_header\n1\n")
    with pytest.raises(L.LcrError):
        L.read_ply(tmp_path / "short.ply")
    with pytest.raises(L.LcrError):
        L.read_ply(tmp_path / "missing.ply")


def test_large_text_round_trip_uses_the_parallel_form(tmp_path):
    pts = random_cloud(150_000, 5)
    pts["normal_y"][::1000] = np.nan
    L.write_ply(tmp_path / "big.ply", pts, binary=False)
    back = L.read_ply(tmp_path / "big.ply")
    for f in FIELDS:
        np.testing.assert_array_equal(back[f], pts[f], err_msg=f)


def test_text_instances_split_over_lines(tmp_path):
    """Any whitespace layout is valid PLY: the token-stream form reads it."""
    text = ("ply\nformat ascii 1.0\nelement vertex 2\nproperty float x\nproperty float y\nproperty float z\n"
            "end_header\n1.5\n2.5 3.5 -4\n+5e-1\n6\n")
    (tmp_path / "s.ply").write_text(text)
    p = L.read_ply(tmp_path / "s.ply")
    np.testing.assert_array_equal(p["x"], np.float32([1.5, -4.0]))
    np.testing.assert_array_equal(p["y"], np.float32([2.5, 0.5]))
    np.testing.assert_array_equal(p["z"], np.float32([3.5, 6.0]))


def _meshlab_header(n: int, fmt: str) -> bytes:
    """The layout meshlabserver writes between the tools in alignment.sh
    (:99-100, :110): VCG vertex properties with alpha, and an empty face list."""
    return (f"ply\nformat {fmt} 1.0\ncomment VCGLIB generated\nelement vertex {n}\n"
            "property float x\nproperty float y\nproperty float z\n"
            "property float nx\nproperty float ny\nproperty float nz\n"
            "property uchar red\nproperty uchar green\nproperty uchar blue\nproperty uchar alpha\n"
            "element face 0\nproperty list uchar int vertex_indices\nend_header\n").encode()


@pytest.mark.parametrize("fmt", ["binary_little_endian", "binary_big_endian"])
def test_meshlab_vertex_layout(tmp_path, fmt):
    n = 7
    rng = np.random.default_rng(5)
    xyz = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    nrm = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    rgba = rng.integers(0, 256, (n, 4)).astype(np.uint8)
    e = "<f4" if fmt == "binary_little_endian" else ">f4"
    body = b"".join(xyz[i].astype(e).tobytes() + nrm[i].astype(e).tobytes() + rgba[i].tobytes() for i in range(n))
    (tmp_path / "m.ply").write_bytes(_meshlab_header(n, fmt) + body)
    p = L.read_ply(tmp_path / "m.ply")
    assert len(p) == n
    np.testing.assert_array_equal(np.c_[p["x"], p["y"], p["z"]], xyz)
    np.testing.assert_array_equal(np.c_[p["normal_x"], p["normal_y"], p["normal_z"]], nrm)
    np.testing.assert_array_equal(np.c_[p["r"], p["g"], p["b"]], rgba[:, :3])
