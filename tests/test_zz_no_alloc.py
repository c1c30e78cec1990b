"""lcr_backproject_into (the allocation-free back-projection) against the
allocating entry point lcr_backproject_device, on two calls in a row through
the same static scratch.  Collected last; also passes alone."""
from __future__ import annotations

import numpy as np
import pytest

from lowcost3dreconstruction_gb300 import _lib as L
from lowcost3dreconstruction_gb300 import synthetic as S
from lowcost3dreconstruction_gb300.core import Context, LcrError

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FIELDS = ("x", "y", "z", "normal_x", "normal_y", "normal_z", "curvature", "r", "g", "b")


def _records(buf: "torch.Tensor", n: int) -> np.ndarray:
    from oracle.oracle import POINT_DTYPE
    raw = buf[: 48 * n].cpu().numpy()
    return raw.view(POINT_DTYPE) if n else np.zeros(0, dtype=POINT_DTYPE)


def _into(ctx: Context, frames: np.ndarray, params) -> np.ndarray:
    d_in = torch.from_numpy(frames.view(np.uint8).reshape(-1).copy()).cuda()
    cap = params.width * params.height
    d_pts = torch.zeros(48 * cap, dtype=torch.uint8, device="cuda")
    d_cnt = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    ctx.backproject_into(d_in.data_ptr(), params, d_pts.data_ptr(), cap, d_cnt.data_ptr())
    ctx.synchronize()
    n = int(d_cnt.item())
    assert 0 <= n <= cap
    return _records(d_pts, n)


def _device(ctx: Context, frames: np.ndarray, params) -> np.ndarray:
    d_in = torch.from_numpy(frames.view(np.uint8).reshape(-1).copy()).cuda()
    torch.cuda.synchronize()
    return ctx.backproject_device(d_in.data_ptr(), params).download()


def _same(a: np.ndarray, b: np.ndarray) -> None:
    assert len(a) == len(b)
    for f in FIELDS:
        x, y = a[f], b[f]
        if x.dtype.kind == "f":
            np.testing.assert_array_equal(x.view(np.uint32), y.view(np.uint32), err_msg=f)
        else:
            np.testing.assert_array_equal(x, y, err_msg=f)


def test_into_matches_allocating_entry_twice():
    pr = S.config1_pair(2)
    with Context(0) as ctx:
        v1 = ctx.depth_params(L.KINECT_V1, 640, 480, frames=10, scale=0.001, depth_max=4000.0, normals=True)
        # two calls in a row on the same scratch: source burst, then target burst
        for frames in (pr.src_frames, pr.tgt_frames):
            frames = np.ascontiguousarray(frames, dtype=np.uint16)
            a = _into(ctx, frames, v1)
            b = _device(ctx, frames, v1)
            assert len(a) > 200_000
            _same(a, b)


def test_into_kinect_v2_and_single_frame():
    cam = S.KINECT_V2
    d = S.raycast(S.sphere_on_cube_room(), cam)
    fr = S.kinect_frames(d, 3, np.random.default_rng(9), as_float=True).astype(np.float32)
    with Context(0) as ctx:
        v2 = ctx.depth_params(L.KINECT_V2, 512, 424, frames=3, fx=365.0, fy=365.0, cx=255.5, cy=211.5,
                              depth_min=500, depth_max=2500, roi=(20, 490, 10, 400), scale=1000.0 / 4500.0,
                              normals=False)
        _same(_into(ctx, fr, v2), _device(ctx, fr, v2))
        one = ctx.depth_params(L.KINECT_V2, 512, 424, frames=1, fx=365.0, fy=365.0, cx=255.5, cy=211.5,
                               depth_min=500, depth_max=2500, scale=1.0, normals=False)
        f0 = np.ascontiguousarray(fr[0])
        _same(_into(ctx, f0, one), _device(ctx, f0, one))


def test_into_pinhole_float_burst():
    """LCR_DEPTH_PINHOLE_F32 (the Kinect v2 super-resolution cloud): a fused
    float burst with normals, through both entry points."""
    cam = S.KINECT_V2
    d = S.raycast(S.sphere_on_cube_room(), cam)
    fr = S.kinect_frames(d, 3, np.random.default_rng(11), as_float=True).astype(np.float32)
    with Context(0) as ctx:
        p = ctx.depth_params(L.PINHOLE_F32, 512, 424, frames=3, fx=365.531799, fy=365.531799, cx=256.136810,
                             cy=206.013901, depth_min=500, depth_max=2500, scale=1.0, normals=True)
        a = _into(ctx, fr, p)
        assert len(a) > 10_000
        _same(a, _device(ctx, fr, p))


def test_into_truncates_at_capacity_and_reports_the_count():
    pr = S.config1_pair(2)
    frames = np.ascontiguousarray(pr.src_frames[0], dtype=np.uint16)
    with Context(0) as ctx:
        p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=1, scale=0.001, depth_max=4000.0)
        full = _device(ctx, frames, p)
        d_in = torch.from_numpy(frames.view(np.uint8).reshape(-1).copy()).cuda()
        cap = 1000
        d_pts = torch.zeros(48 * cap, dtype=torch.uint8, device="cuda")
        d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        ctx.backproject_into(d_in.data_ptr(), p, d_pts.data_ptr(), cap, d_cnt.data_ptr())
        ctx.synchronize()
        assert int(d_cnt.item()) == len(full)
        _same(_records(d_pts, cap), full[:cap])


def test_into_rejects_images_above_its_scratch():
    with Context(0) as ctx:
        p = ctx.depth_params(L.KINECT_V1, 641, 480, frames=1)
        d_in = torch.zeros(641 * 480, dtype=torch.int16, device="cuda")
        d_pts = torch.zeros(48, dtype=torch.uint8, device="cuda")
        d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        with pytest.raises(LcrError) as e:
            ctx.backproject_into(d_in.data_ptr(), p, d_pts.data_ptr(), 1, d_cnt.data_ptr())
        assert e.value.status == L.INVALID_ARG
        assert "scratch" in str(e.value)


def test_into_rejects_misaligned_outputs():
    """The records are written as 16-byte vectors: a point buffer that is not
    16-byte aligned (or a count that is not 4-byte aligned) is refused on the
    host, before any launch."""
    with Context(0) as ctx:
        p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=1)
        d_in = torch.zeros(640 * 480, dtype=torch.int16, device="cuda")
        d_pts = torch.zeros(48 * 16 + 16, dtype=torch.uint8, device="cuda")
        d_cnt = torch.zeros(2, dtype=torch.int32, device="cuda")
        for pts_off, cnt_off in ((4, 0), (0, 2)):
            with pytest.raises(LcrError) as e:
                ctx.backproject_into(d_in.data_ptr(), p, d_pts.data_ptr() + pts_off, 16, d_cnt.data_ptr() + cnt_off)
            assert e.value.status == L.INVALID_ARG and "aligned" in str(e.value)
