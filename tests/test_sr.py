"""Super-resolution front end (capture/super_resolution/super_resolution.cpp:
236-314): ECC registration, warp, nearest upsampling, ZE-mean, Lanczos-4.

CPU: the oracle's pieces (Lanczos weights, smoothing, ECC on a known
motion).  GPU: the library against the oracle on a synthetic burst whose
frames are known affine motions of one smooth depth scene: recovered warps
close to the truth and to the oracle's, the fused image equal to the
oracle's within one unit of rounding."""
from __future__ import annotations

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
