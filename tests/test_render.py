"""Synthetic depth images (lcr_synthetic_depth): the objects of
lcr_synthetic_pairs seen by a Kinect v1 or v2 camera.  Back-projecting a
rendered image with the matching model must put every point on the object's
surface (checked against dense noise-free surface samples of the same view),
the transforms must be the generator's, and distance must scale the point
count as 1/z^2."""
from __future__ import annotations

import numpy as np
import pytest

from lowcost3dreconstruction_gb300 import _lib as L
from lowcost3dreconstruction_gb300.core import xyz_of

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
cKDTree = pytest.importorskip("scipy.spatial").cKDTree

V1 = dict(model=L.KINECT_V1, width=640, height=480, fx=525.0, fy=525.0, cx=319.5, cy=239.5)
V2 = dict(model=L.KINECT_V2, width=512, height=424, fx=365.0, fy=365.0, cx=255.5, cy=211.5)


def _render(ctx, seed, npairs, cam, distance=None, noise=False):
    pix = cam["width"] * cam["height"]
    dt = torch.int16 if cam["model"] == L.KINECT_V1 else torch.float32
    buf = torch.zeros(2 * npairs * pix, dtype=dt, device="cuda")
    torch.cuda.synchronize()
    T = ctx.synthetic_depth(seed, npairs, cam["model"], cam["width"], cam["height"], cam["fx"], cam["fy"], cam["cx"],
                            cam["cy"], buf.data_ptr(), distance=distance, noise=noise)
    return buf, T


def _clouds(ctx, buf, npairs, cam):
    pix = cam["width"] * cam["height"]
    p = ctx.depth_params(cam["model"], cam["width"], cam["height"], frames=1, fx=cam["fx"], fy=cam["fy"],
                         cx=cam["cx"], cy=cam["cy"], scale=0.001 if cam["model"] == L.KINECT_V1 else 1.0,
                         depth_max=100000.0, normals=False)
    es = buf.element_size()
    return [ctx.backproject_device(buf.data_ptr() + v * pix * es, p) for v in range(2 * npairs)]


@pytest.mark.parametrize("cam", [V1, V2], ids=["kinect_v1", "kinect_v2"])
def test_rendered_points_lie_on_the_surface(ctx, cam):
    seed, n = 77, 3
    buf, T = _render(ctx, seed, n, cam)
    src, tgt, T2 = ctx.synthetic_pairs(seed, n, 200_000, noise=False)
    np.testing.assert_array_equal(T, T2)
    clouds = _clouds(ctx, buf, n, cam)
    for i in range(n):
        for view, dense in ((0, src[i]), (1, tgt[i])):
            pts = xyz_of(clouds[2 * i + view].download()).astype(np.float64)
            assert len(pts) > 2000
            d, _ = cKDTree(xyz_of(dense.download()).astype(np.float64)).query(pts)
            assert np.median(d) < 1e-3 and np.percentile(d, 95) < 2.5e-3, (i, view, np.median(d),
                                                                            np.percentile(d, 95))


def test_distance_scales_the_point_count(ctx):
    seed, n = 91, 4
    near, _ = _render(ctx, seed, n, V1, distance=np.full(n, 1.0, np.float32))
    far, _ = _render(ctx, seed, n, V1, distance=np.full(n, 2.0, np.float32))
    a = [len(c) for c in _clouds(ctx, near, n, V1)]
    b = [len(c) for c in _clouds(ctx, far, n, V1)]
    ratio = np.array(b, np.float64) / np.array(a, np.float64)
    assert np.all((ratio > 0.18) & (ratio < 0.32)), ratio


def test_noise_follows_the_kinect_model(ctx):
    seed, n = 5, 2
    clean, _ = _render(ctx, seed, n, V2)
    noisy, _ = _render(ctx, seed, n, V2, noise=True)
    c, z = clean.cpu().numpy(), noisy.cpu().numpy()
    m = c > 0
    assert np.array_equal(m, z > 0)
    r = (z[m] - c[m]) / (1.5 * (c[m] / 1000.0) ** 2)
    assert abs(r.mean()) < 0.02 and 0.95 < r.std() < 1.05


def test_render_rejects_bad_arguments(ctx):
    buf = torch.zeros(16, dtype=torch.int16, device="cuda")
    with pytest.raises(L.LcrError) as e:
        ctx.synthetic_depth(1, 1, 7, 4, 2, 1.0, 1.0, 0.0, 0.0, buf.data_ptr())
    assert e.value.status == L.INVALID_ARG
    with pytest.raises(L.LcrError):
        ctx.synthetic_depth(1, 1, L.KINECT_V1, 4, 2, 1.0, 1.0, 0.0, 0.0, buf.data_ptr(),
                            distance=np.array([0.01], np.float32))


def test_turntable_views_turn_about_the_vertical_axis(ctx):
    """lcr_synthetic_turntable: view 0 is the source view of the seed's pair 0,
    image for image, and view j is the object turned by j * step about its
    vertical axis through its centre."""
    import math
    seed, views, step = 61, 5, 10.0
    pix = V1["width"] * V1["height"]
    buf = torch.zeros(views * pix, dtype=torch.int16, device="cuda")
    torch.cuda.synchronize()
    P = ctx.synthetic_turntable(seed, views, step, L.KINECT_V1, V1["width"], V1["height"], V1["fx"], V1["fy"],
                                V1["cx"], V1["cy"], buf.data_ptr(), distance=1.0).astype(np.float64)
    pair, _ = _render(ctx, seed, 1, V1, distance=np.array([1.0], np.float32), noise=True)
    np.testing.assert_array_equal(buf[:pix].cpu().numpy(), pair[:pix].cpu().numpy())
    for j in range(1, views):
        Tj = P[j] @ np.linalg.inv(P[0])
        c = np.clip((np.trace(Tj[:3, :3]) - 1) / 2, -1, 1)
        assert abs(math.degrees(math.acos(c)) - step * j) < 1e-3
        # the axis is the camera's y axis, and the object's centre stays put
        assert abs(abs(Tj[1, 1]) - 1.0) < 1e-6
        np.testing.assert_allclose(P[j][:3, 3], P[0][:3, 3], atol=1e-6)
    # consecutive views back-project into clouds that overlap after the known motion
    prm = ctx.depth_params(L.KINECT_V1, V1["width"], V1["height"], scale=0.001, depth_max=9000.0, normals=False)
    a = xyz_of(ctx.backproject_device(buf.data_ptr(), prm).download()).astype(np.float64)
    b = xyz_of(ctx.backproject_device(buf.data_ptr() + 2 * pix, prm).download()).astype(np.float64)
    T10 = P[0] @ np.linalg.inv(P[1])
    bb = b @ T10[:3, :3].T + T10[:3, 3]
    d, _ = cKDTree(a).query(bb)
    assert np.median(d) < 2e-3
