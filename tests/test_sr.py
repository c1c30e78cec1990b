"""Super-resolution front end (capture/super_resolution/super_resolution.cpp:
236-314): ECC registration, warp, nearest upsampling, ZE-mean, Lanczos-4.

CPU: the oracle's pieces (Lanczos weights, smoothing, ECC on a known
motion).  GPU: the library against the oracle on a synthetic burst whose
frames are known affine motions of one smooth depth scene: recovered warps
close to the truth and to the oracle's, the fused image equal to the
oracle's within one unit of rounding."""
from __future__ import annotations

import struct
import subprocess
import zlib
from pathlib import Path

import numpy as np
import pytest

from oracle import sr as O


def depth_scene(x, y):
    return (1000 + 120 * np.sin(x / 9.0) * np.cos(y / 7.0) + 60 * np.exp(-((x - 50) ** 2 + (y - 40) ** 2) / 200.0)
            + 0.8 * x - 0.5 * y)


def burst(h=72, w=96, F=4, seed=0, holes=True):
    """Frame f samples the scene at B_f (x, y): ECC should recover inv(B_f)."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)
    frames, truth = [], []
    for f in range(F):
        if f == 0:
            B = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1]], np.float64)
        else:
            a = np.deg2rad(rng.uniform(-0.4, 0.4))
            B = np.array([[np.cos(a), -np.sin(a), rng.uniform(-0.8, 0.8)],
                          [np.sin(a), np.cos(a), rng.uniform(-0.8, 0.8)], [0, 0, 1]])
        X = B[0, 0] * x + B[0, 1] * y + B[0, 2]
        Y = B[1, 0] * x + B[1, 1] * y + B[1, 2]
        d = depth_scene(X, Y) + rng.normal(0, 0.3, x.shape)
        if holes:
            d[rng.random(d.shape) < 0.01] = 0
        frames.append(np.clip(np.rint(d), 0, 65535).astype(np.uint16))
        truth.append(np.linalg.inv(B)[:2])
    return np.stack(frames), np.stack(truth)


# ------------------------------------------------------------------ CPU
def test_oracle_lanczos_weights():
    for t in (0.0, 0.25, 0.5, 0.9):
        w = O.lanczos4_weights(t)
        assert abs(float(w.sum()) - 1) < 1e-6
    np.testing.assert_array_equal(O.lanczos4_weights(0.0), np.eye(8, dtype=np.float32)[3])


def test_oracle_filters_agree_with_scipy():
    """The oracle's smoothing, gradients and bilinear sampling against
    scipy.ndimage, an independent implementation of the same operations
    (reflect-101 is scipy's 'mirror'; the zero border is 'constant', 0)."""
    nd = pytest.importorskip("scipy.ndimage")
    img = burst(F=1, seed=12, holes=True)[0][0].astype(np.float32)
    s = 1.1
    g = np.array([np.exp(-4 / (2 * s * s)), np.exp(-1 / (2 * s * s)), 1.0, np.exp(-1 / (2 * s * s)),
                  np.exp(-4 / (2 * s * s))])
    g /= g.sum()
    want = nd.correlate1d(nd.correlate1d(img.astype(np.float64), g, axis=1, mode="mirror"), g, axis=0, mode="mirror")
    np.testing.assert_allclose(O.gauss5(img), want, rtol=1e-6, atol=1e-3)
    gx, gy = O.grad(img)
    np.testing.assert_allclose(gx[:, 1:-1], np.gradient(img.astype(np.float64), axis=1)[:, 1:-1], atol=1e-3)
    np.testing.assert_allclose(gy[1:-1], np.gradient(img.astype(np.float64), axis=0)[1:-1], atol=1e-3)
    rng = np.random.default_rng(13)
    u = rng.uniform(0, img.shape[1] - 1, 500).astype(np.float32)
    v = rng.uniform(0, img.shape[0] - 1, 500).astype(np.float32)
    ref = nd.map_coordinates(img.astype(np.float64), [v, u], order=1, mode="constant", cval=0.0)
    np.testing.assert_allclose(O.bilinear(img, u, v), ref, rtol=1e-6, atol=1e-3)


def test_oracle_lanczos_reproduces_a_linear_ramp():
    """Downsampling by 4 samples at p = 4 o + 1.5, where the normalised
    Lanczos-4 weights are symmetric: a linear ramp comes out as its value at
    p (away from the clamped borders) -- a property, not a restatement."""
    H, W = 64, 96
    y, x = np.mgrid[0:H, 0:W].astype(np.float64)
    ramp = (100 + 3 * x - 2 * y).astype(np.float32)
    out = O.lanczos_down(ramp, 4)
    oy, ox = np.mgrid[0:H // 4, 0:W // 4].astype(np.float64)
    want = 100 + 3 * (4 * ox + 1.5) - 2 * (4 * oy + 1.5)
    np.testing.assert_allclose(out[1:-1, 1:-1], want[1:-1, 1:-1], atol=2e-3)


@pytest.mark.parametrize("kind", ["holed", "clean", "float"])
def test_c_oracle_agrees_with_the_numpy_oracle(kind):
    """oracle/sr_oracle.cpp (the CPU baseline) against oracle/sr.py: the same
    iterations and warps; the fused image within one unit (float: 1e-3)."""
    from oracle import oracle as OC
    frames, _ = burst(F=4, seed=1 if kind == "holed" else 3, holes=kind == "holed")
    if kind == "float":
        frames = frames.astype(np.float32) + np.float32(0.25)
    a, wa, ia = O.super_resolve(frames, 4, 60, 1e-10)
    b, wb, ib = OC.super_resolve(frames, 4, 60, 1e-10)
    np.testing.assert_array_equal(ia, ib)
    np.testing.assert_allclose(wa, wb, atol=1e-6)
    if kind == "float":
        np.testing.assert_allclose(a, b, atol=1e-3)
    else:
        assert np.abs(a.astype(np.int64) - b.astype(np.int64)).max() <= 1


def test_oracle_ecc_recovers_a_known_motion():
    frames, truth = burst(F=2, holes=False)
    blur = O.gauss5(frames.astype(np.float32))
    gx, gy = O.grad(blur)
    m, it = O.ecc_affine(blur[0], blur[1], gx[1], gy[1], 100, 1e-10)
    np.testing.assert_allclose(m[:, 2], truth[1][:, 2], atol=0.05)
    np.testing.assert_allclose(m[:, :2], truth[1][:, :2], atol=2e-3)


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_super_resolve_matches_oracle(ctx):
    """A burst with 1% missing pixels (zeros): like the reference, which passes
    no mask to the registration, zeros take part as intensities -- the GPU
    and the oracle must agree, whatever the holes do to the motion."""
    frames, _ = burst(F=4, seed=1)
    out, warps, mm, its = ctx.super_resolve(frames, factor=4, ecc_iterations=60, ecc_epsilon=1e-10)
    want, wwarps, wits = O.super_resolve(frames, 4, 60, 1e-10)
    nz = frames[frames > 0]
    assert mm == (float(nz.min()), float(nz.max()))
    np.testing.assert_array_equal(warps[0], np.float32([[1, 0, 0], [0, 1, 0]]))
    for f in range(1, 4):
        np.testing.assert_allclose(warps[f], wwarps[f], atol=2e-3)
    diff = np.abs(out.astype(np.int64) - want.astype(np.int64))
    assert np.mean(diff <= 1) > 0.995
    assert np.mean((out == 0) != (want == 0)) < 1e-3


@pytest.mark.gpu
def test_ecc_recovers_known_motions(ctx):
    frames, truth = burst(F=6, seed=3, holes=False)
    _, warps, _, its = ctx.super_resolve(frames, factor=4, ecc_iterations=100, ecc_epsilon=1e-10)
    assert its[0] == 0 and np.all(its[1:] >= 1)
    for f in range(1, 6):
        np.testing.assert_allclose(warps[f][:, 2], truth[f][:, 2], atol=0.05)
        np.testing.assert_allclose(warps[f][:, :2], truth[f][:, :2], atol=2e-3)


@pytest.mark.gpu
def test_super_resolve_single_frame_is_a_lanczos_round_trip(ctx):
    """One frame: no registration, the fused image is the frame upsampled and
    resampled back (a block-constant image through Lanczos-4)."""
    frames, _ = burst(F=1, seed=2, holes=False)
    out, warps, _, its = ctx.super_resolve(frames, factor=4)
    want, _, _ = O.super_resolve(frames, 4)
    assert its[0] == 0
    assert np.mean(np.abs(out.astype(np.int64) - want.astype(np.int64)) <= 1) > 0.999
    assert np.mean(np.abs(out.astype(np.int64) - frames[0].astype(np.int64))) < 3.0


# ------------------------------------------------------------------ the tool
# capture/super_resolution/super_resolution.cpp: flags and messages (:142-211),
# <name>_burst_<view>_<i>.png in, <name>_srdepth_<view>.png and
# <name>_srmesh_<view>.ply out.
BIN = Path(__file__).resolve().parents[1] / "lowcost3dreconstruction_gb300" / "bin"


def _paeth(a: int, b: int, c: int) -> int:
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    return a if pa <= pb and pa <= pc else (b if pb <= pc else c)


def _write_png(path, rows: bytes, w: int, h: int, depth: int, ctype: int, bpp: int) -> None:
    """PNG of h rows of w * bpp bytes, row y filtered with filter type y % 5
    so that the tool's decoder meets every scanline filter."""
    stride = w * bpp
    raw = bytearray()
    prev = bytes(stride)
    for y in range(h):
        row = rows[y * stride:(y + 1) * stride]
        ft = y % 5
        out = bytearray([ft])
        for i in range(stride):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[ft]
            out.append((row[i] - pred) & 255)
        raw += out
        prev = row

    def chunk(t: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)
    png = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    png += chunk(b"IDAT", zlib.compress(bytes(raw), 6)) + chunk(b"IEND", b"")
    Path(path).write_bytes(png)


def write_png16(path, img: np.ndarray) -> None:
    h, w = img.shape
    _write_png(path, img.astype(">u2").tobytes(), w, h, 16, 0, 2)


def write_png_float(path, img: np.ndarray) -> None:
    """A float depth image as the Kinect v2 tools store it: each float's
    little-endian bytes b0..b3 are an OpenCV BGRA pixel, i.e. the PNG's RGBA
    pixel (b2, b1, b0, b3)."""
    h, w = img.shape
    b = np.ascontiguousarray(img, dtype="<f4").view(np.uint8).reshape(h, w, 4)
    _write_png(path, np.ascontiguousarray(b[..., [2, 1, 0, 3]]).tobytes(), w, h, 8, 6, 4)


def _read_png(path):
    """(unfiltered bytes [h][stride], w, h, depth, ctype) of the tool's
    output: filter type 0 on every row."""
    data = Path(path).read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h, depth, ctype = 8, b"", 0, 0, 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        t, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(t + body) & 0xFFFFFFFF
        if t == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
        elif t == b"IDAT":
            idat += body
        pos += 12 + n
    bpp = (1 if ctype == 0 else 4) * depth // 8
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + bpp * w)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].copy(), w, h, depth, ctype


def read_png16(path) -> np.ndarray:
    rows, w, h, depth, ctype = _read_png(path)
    assert depth == 16 and ctype == 0
    return rows.view(">u2").astype(np.uint16).reshape(h, w)


def read_png_float(path) -> np.ndarray:
    rows, w, h, depth, ctype = _read_png(path)
    assert depth == 8 and ctype == 6
    px = rows.reshape(h, w, 4)[..., [2, 1, 0, 3]]
    return np.ascontiguousarray(px).view("<f4").reshape(h, w).astype(np.float32)


def run_tool(*args, cwd, tool="super_resolution"):
    return subprocess.run([str(BIN / tool), *map(str, args)], capture_output=True, text=True,
                          timeout=300, cwd=cwd)


@pytest.fixture(scope="module")
def sr_tool():
    from lowcost3dreconstruction_gb300 import build
    build.build_lib()
    build.build_tools()
    if not (BIN / "super_resolution").exists() or not (BIN / "super_resolution_kv2").exists():
        pytest.skip("the super-resolution tools need zlib headers")


def test_png_writer_reader_round_trip(tmp_path):
    img = np.random.default_rng(0).integers(0, 65536, (7, 11)).astype(np.uint16)
    write_png16(tmp_path / "a.png", img)
    data = (tmp_path / "a.png").read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n" and b"IHDR" in data


def test_png_float_round_trip(tmp_path):
    img = np.random.default_rng(1).uniform(500, 1500, (5, 9)).astype(np.float32)
    write_png_float(tmp_path / "f.png", img)
    data = (tmp_path / "f.png").read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"


@pytest.mark.parametrize("tool", ["super_resolution", "super_resolution_kv2"])
def test_tool_help_and_usage_errors(sr_tool, tmp_path, tool):
    r = run_tool("-h", cwd=tmp_path, tool=tool)
    assert r.returncode == 0
    for f in ("--capture_name", "--capture_step", "--num_captures", "--sr_size", "--resample_factor",
              "--view_angle", "--top", "--bottom"):
        assert f in r.stdout, f
    assert "(=artefact)" in r.stdout and "(=16)" in r.stdout and "(=4)" in r.stdout
    r = run_tool("-f", "0", cwd=tmp_path, tool=tool)
    assert r.returncode == 255 and "must be bigger than zero" in r.stdout
    r = run_tool("-a", "20", "-t", cwd=tmp_path, tool=tool)
    assert r.returncode == 255 and "can not be used together" in r.stdout
    r = run_tool("-a", "20", "-n", "missing", cwd=tmp_path, tool=tool)
    assert r.returncode == 255 and "Image can not be read: missing_burst_20_0.png" in r.stdout


def test_kv2_tool_rejects_a_grayscale_burst(sr_tool, tmp_path):
    write_png16(tmp_path / "g_burst_0_0.png", np.ones((4, 4), np.uint16))
    r = run_tool("-n", "g", "-a", "0", "-z", "1", cwd=tmp_path, tool="super_resolution_kv2")
    assert r.returncode == 255 and "Image can not be read: g_burst_0_0.png" in r.stdout


def test_oracle_kv2_leaves_uncovered_pixels_zero():
    frames, _ = burst(F=2, seed=4, holes=False)
    f = frames.astype(np.float32)
    f[:, 10:30, 20:40] = 0  # no frame covers the middle of this square
    out, _, _ = O.super_resolve(f, 4, 5, 1e-10)
    assert out.dtype == np.float32 and np.all(np.isfinite(out))
    assert np.all(out[15:25, 25:35] == 0)


@pytest.mark.gpu
def test_tool_writes_the_fused_depth_and_cloud(sr_tool, tmp_path, ctx):
    from lowcost3dreconstruction_gb300 import _lib as L
    frames, _ = burst(h=48, w=64, F=4, seed=5, holes=False)
    for i, f in enumerate(frames):
        write_png16(tmp_path / f"obj_burst_top_{i}.png", f)
    r = run_tool("-n", "obj", "-t", "-z", 4, "-f", 4, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    want, warps, mm, _ = ctx.super_resolve(frames, factor=4)
    assert f"Observed Global Min: {mm[0]:.0f}" in r.stdout
    assert f"Observed Global Max: {mm[1]:.0f}" in r.stdout
    assert "View(top) Alignment 3-> 0 = [" in r.stdout
    got = read_png16(tmp_path / "obj_srdepth_top.png")
    np.testing.assert_array_equal(got, want)
    pts = L.read_ply(tmp_path / "obj_srmesh_top.ply")
    p = L.DepthParams(L.KINECT_V1, 64, 48, 1, 572.882768, 542.739980, 314.649173, 240.160459, mm[0], mm[1],
                      0, 63, 0, 47, 1.0, 1, 128, 128, 128, 0)
    cloud = ctx.backproject(want, p).download()
    assert len(pts) == len(cloud) > 0
    np.testing.assert_allclose(pts["x"], cloud["x"], rtol=1e-6, atol=1e-4)
    np.testing.assert_allclose(pts["z"], cloud["z"], rtol=1e-6, atol=1e-4)
    assert (tmp_path / "obj_srmesh_top.ply").read_bytes().startswith(b"ply\nformat ascii")


def smooth_burst(F=3, seed=21):
    """640 x 480 frames of a smooth scene under small rigid motions (the
    registration settles in a few iterations at eps 1e-12)."""
    h, w = 480, 640
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:h, 0:w].astype(np.float64)

    def scene(X, Y):
        return (1000 + 120 * np.sin(X / 27.0) * np.cos(Y / 21.0)
                + 60 * np.exp(-((X - 320) ** 2 + (Y - 240) ** 2) / 1800.0) + 0.3 * X - 0.2 * Y)
    fr = []
    for f in range(F):
        a = 0.0 if f == 0 else np.deg2rad(rng.uniform(-0.4, 0.4))
        tx, ty = (0.0, 0.0) if f == 0 else rng.uniform(-0.8, 0.8, 2)
        X = np.cos(a) * x - np.sin(a) * y + tx
        Y = np.sin(a) * x + np.cos(a) * y + ty
        fr.append(np.clip(np.rint(scene(X, Y) + rng.normal(0, 0.3, x.shape)), 0, 65535).astype(np.uint16))
    return np.stack(fr)


@pytest.mark.gpu
def test_ecc_stops_when_the_coefficient_settles(ctx):
    """At eps 1e-12 the stopping test needs the correlation coefficient exact
    to ~1e-13 between iterations: the oracle (FP64 throughout) stops within
    ten iterations here, and so must the GPU."""
    frames = smooth_burst()
    _, warps, _, its = ctx.super_resolve(frames)
    _, wwarps, wits = O.super_resolve(frames)
    assert np.all(wits[1:] < 10)
    assert np.all(its[1:] < 20), its
    np.testing.assert_allclose(warps, wwarps, atol=5e-5)


# ------------------------------------------------------------------ Kinect v2
@pytest.mark.gpu
def test_super_resolve_f32_matches_the_uint16_path(ctx):
    """Float frames holding whole millimetres take the same arithmetic as the
    uint16 frames: the same warps and iterations, and the float result
    rounds to the uint16 result (every pixel is covered by frame 0)."""
    frames, _ = burst(F=4, seed=6, holes=False)
    out16, w16, mm16, it16 = ctx.super_resolve(frames, ecc_iterations=50, ecc_epsilon=1e-10)
    outf, wf, mmf, itf = ctx.super_resolve(frames.astype(np.float32), ecc_iterations=50, ecc_epsilon=1e-10)
    assert outf.dtype == np.float32 and out16.dtype == np.uint16
    np.testing.assert_array_equal(wf, w16)
    np.testing.assert_array_equal(itf, it16)
    assert mmf == mm16
    np.testing.assert_array_equal(np.clip(np.rint(outf), 0, 65535).astype(np.uint16), out16)


@pytest.mark.gpu
def test_super_resolve_f32_matches_oracle(ctx):
    rng = np.random.default_rng(8)
    frames, _ = burst(F=3, seed=7, holes=False)
    f = (frames.astype(np.float32) + rng.uniform(-0.5, 0.5, frames.shape)).astype(np.float32)
    out, warps, mm, _ = ctx.super_resolve(f, ecc_iterations=40, ecc_epsilon=1e-10)
    want, wwarps, _ = O.super_resolve(f, 4, 40, 1e-10)
    pos = f[f > 0]
    assert mm == (float(pos.min()), float(pos.max()))
    for k in range(1, 3):
        np.testing.assert_allclose(warps[k], wwarps[k], atol=2e-3)
    assert np.mean(np.abs(out - want) <= 0.05) > 0.995


@pytest.mark.gpu
def test_pinhole_f32_backprojection_equals_v1_on_whole_millimetres(ctx):
    """LCR_DEPTH_PINHOLE_F32 (super_resolution_kv2.cpp save_ply) on float
    depth that holds whole millimetres: the same points and normals as the
    uint16 model, bit for bit."""
    from lowcost3dreconstruction_gb300 import _lib as L
    frames, _ = burst(h=48, w=64, F=1, seed=9, holes=True)
    d = frames[0]
    args = (64, 48, 1, 365.531799, 365.531799, 256.136810, 206.013901, 900.0, 1200.0, 0, 63, 0, 47, 1.0, 1,
            128, 128, 128, 0)
    a = ctx.backproject(d, L.DepthParams(L.KINECT_V1, *args)).download()
    b = ctx.backproject(d.astype(np.float32), L.DepthParams(L.PINHOLE_F32, *args)).download()
    assert len(a) == len(b) > 0
    for k in a.dtype.names:
        np.testing.assert_array_equal(a[k], b[k])


@pytest.mark.gpu
def test_kv2_tool_writes_the_fused_depth_and_cloud(sr_tool, tmp_path, ctx):
    from lowcost3dreconstruction_gb300 import _lib as L
    rng = np.random.default_rng(10)
    frames, _ = burst(h=48, w=64, F=4, seed=11, holes=False)
    f = (frames.astype(np.float32) + rng.uniform(-0.5, 0.5, frames.shape)).astype(np.float32)
    for i, fr in enumerate(f):
        write_png_float(tmp_path / f"obj_burst_40_{i}.png", fr)
    r = run_tool("-n", "obj", "-a", 40, "-z", 4, cwd=tmp_path, tool="super_resolution_kv2")
    assert r.returncode == 0, r.stdout + r.stderr
    want, _, mm, _ = ctx.super_resolve(f)
    assert f"Observed Global Min: {mm[0]:.0f}" in r.stdout
    assert "View(40) Alignment 3-> 0 = [" in r.stdout
    np.testing.assert_array_equal(read_png_float(tmp_path / "obj_srdepth_40.png"), want)
    pts = L.read_ply(tmp_path / "obj_srmesh_40.ply")
    p = L.DepthParams(L.PINHOLE_F32, 64, 48, 1, 365.531799, 365.531799, 256.136810, 206.013901, mm[0], mm[1],
                      0, 63, 0, 47, 1.0, 1, 128, 128, 128, 0)
    cloud = ctx.backproject(want, p).download()
    assert len(pts) == len(cloud) > 0
    np.testing.assert_allclose(pts["z"], cloud["z"], rtol=1e-6, atol=1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("h,w,F,factor", [(5, 7, 3, 4), (1, 9, 2, 4), (33, 130, 4, 1), (40, 40, 2, 3), (24, 20, 1, 16)])
def test_super_resolve_odd_shapes_match_oracle(ctx, h, w, F, factor):
    """Ragged sizes (no multiple of a block, a single row, factor 1 and 16,
    one frame): the same result as the oracle within one unit."""
    frames, _ = burst(h=h, w=w, F=F, seed=h * w + F, holes=False)
    out, warps, mm, its = ctx.super_resolve(frames, factor=factor, ecc_iterations=30, ecc_epsilon=1e-10)
    want, wwarps, wits = O.super_resolve(frames, factor, 30, 1e-10)
    assert out.shape == (h, w) and np.all(its <= 30)
    if h * w < 100:  # a handful of pixels: the registration is too ill-posed to compare paths
        assert mm == (float(frames[frames > 0].min()), float(frames.max()))
        return
    np.testing.assert_allclose(warps, wwarps, atol=2e-3)
    assert np.mean(np.abs(out.astype(np.int64) - want.astype(np.int64)) <= 1) > 0.99


@pytest.mark.gpu
def test_super_resolve_all_zero_burst(ctx):
    """No depth anywhere: the registration stops at once (singular system),
    the range is (0, 0) and the fused image is all zero, as the oracle says."""
    frames = np.zeros((3, 24, 32), np.uint16)
    out, warps, mm, its = ctx.super_resolve(frames)
    want, wwarps, wits = O.super_resolve(frames)
    assert mm == (0.0, 0.0)
    assert np.all(out == 0) and np.all(want == 0)
    np.testing.assert_array_equal(its, wits)
    np.testing.assert_array_equal(warps, wwarps)


@pytest.mark.gpu
def test_tool_iterates_the_views_and_wraps_the_angle(sr_tool, tmp_path):
    """-c 2 -s 20 fuses views 0 and 20; -a 380 names view 20 (the angle is
    taken modulo 360, super_resolution.cpp:194)."""
    for view in (0, 20):
        frames, _ = burst(h=24, w=32, F=2, seed=20 + view, holes=False)
        for i, f in enumerate(frames):
            write_png16(tmp_path / f"m_burst_{view}_{i}.png", f)
    r = run_tool("-n", "m", "-c", 2, "-s", 20, "-z", 2, cwd=tmp_path)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Step: 20" in r.stdout and "N. of captures: 2" in r.stdout
    for view in (0, 20):
        assert (tmp_path / f"m_srdepth_{view}.png").exists() and (tmp_path / f"m_srmesh_{view}.ply").exists()
    first = (tmp_path / "m_srdepth_20.png").read_bytes()
    (tmp_path / "m_srdepth_20.png").unlink()
    r = run_tool("-n", "m", "-a", 380, "-z", 2, cwd=tmp_path)
    assert r.returncode == 0 and "View angle: 20" in r.stdout
    assert (tmp_path / "m_srdepth_20.png").read_bytes() == first


# ------------------------------------------------------------------ fixtures
GOLD = Path(__file__).resolve().parent / "golden" / "sr_small.npz"


def test_oracle_reproduces_the_committed_fixture():
    """tests/golden/sr_small.npz (made by tests/golden/make_golden.py sr)
    pins the oracle's own outputs on a holed 4-frame burst, uint16 and float."""
    g = np.load(GOLD)
    out, warps, its = O.super_resolve(g["frames"], 4, 30, 1e-10)
    np.testing.assert_array_equal(its, g["iters"])
    np.testing.assert_allclose(warps, g["warps"], atol=1e-6)
    assert np.abs(out.astype(np.int64) - g["fused"].astype(np.int64)).max() <= 1
    outf, warpsf, itsf = O.super_resolve(g["frames_f32"], 4, 30, 1e-10)
    np.testing.assert_array_equal(itsf, g["iters_f32"])
    np.testing.assert_allclose(warpsf, g["warps_f32"], atol=1e-6)
    np.testing.assert_allclose(outf, g["fused_f32"], atol=1e-3)


@pytest.mark.gpu
def test_super_resolve_matches_the_committed_fixture(ctx):
    g = np.load(GOLD)
    for key in ("", "_f32"):
        out, warps, _, _ = ctx.super_resolve(g["frames" + key], ecc_iterations=30, ecc_epsilon=1e-10)
        np.testing.assert_allclose(warps, g["warps" + key], atol=2e-3)
        want = g["fused" + key]
        tol = 1 if key == "" else 0.05
        assert np.mean(np.abs(out.astype(np.float64) - want.astype(np.float64)) <= tol) > 0.99


@pytest.mark.gpu
def test_super_resolve_rejects_bad_arguments(ctx):
    """Invalid sizes and limits come back as LCR_ERR_INVALID_ARG with a
    message, and the context stays usable."""
    from lowcost3dreconstruction_gb300 import _lib as L
    frames, _ = burst(h=16, w=20, F=2, seed=30, holes=False)
    for kw, msg in (({"factor": 0}, "factor"), ({"factor": 17}, "factor"), ({"ecc_iterations": -1}, "ECC"),
                    ({"ecc_epsilon": -1.0}, "ECC")):
        with pytest.raises(L.LcrError) as e:
            ctx.super_resolve(frames, **kw)
        assert e.value.status == L.INVALID_ARG and msg in str(e.value)
    out, _, _, _ = ctx.super_resolve(frames, ecc_iterations=5)
    assert out.shape == (16, 20)
