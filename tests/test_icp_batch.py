"""lcr_icp_batch: all pairs iterate together over one work queue, and every
pair's result is exactly what lcr_icp gives for it alone (fixed-order sums
per pair), whatever the other pairs of the batch are."""
from __future__ import annotations

import numpy as np
import pytest

from lowcost3dreconstruction_gb300 import _lib as L
from lowcost3dreconstruction_gb300 import synthetic as S
from lowcost3dreconstruction_gb300.core import xyz_of
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _same(a, b):
    np.testing.assert_array_equal(a.transform64, b.transform64)
    assert (a.converged, a.iterations, a.state, a.n_correspondences) == \
        (b.converged, b.iterations, b.state, b.n_correspondences)
    assert a.fitness == b.fitness and a.mse == b.mse


@pytest.fixture(scope="module")
def clouds(ctx):
    """Uneven pairs: config-0 clouds at three voxel sizes, plus their normals."""
    pr = S.config0_pair(0)
    prm = O.bp_params(640, 480, scale=0.001, depth_max=4000)
    src = O.backproject_v1(pr.src_frames[0], prm)
    tgt = O.backproject_v1(pr.tgt_frames[0], prm)
    out = []
    for leaf in (0.002, 0.003, 0.005):
        s, _ = O.voxel_grid(src, leaf)
        t, _ = O.voxel_grid(tgt, leaf)
        out.append((ctx.upload(O.normals(s, 20)), ctx.upload(O.normals(t, 20))))
    return out


@pytest.mark.parametrize("p2pl", [False, True])
def test_batch_equals_single_pairs(ctx, clouds, p2pl):
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=40, transformation_epsilon=1e-8,
                         point_to_plane=p2pl)
    # reversed and repeated pairs: sizes and iteration counts differ across the batch
    pairs = clouds + [(t, s) for s, t in clouds] + [clouds[0]]
    single = [ctx.icp(s, t, prm) for s, t in pairs]
    batch = ctx.icp_batch([s for s, _ in pairs], [t for _, t in pairs], prm)
    assert len({r.iterations for r in single}) > 1
    for a, b in zip(batch, single):
        _same(a, b)


def test_batch_guesses_and_a_pair_without_correspondences(ctx, clouds):
    s0, t0 = clouds[1]
    shift = np.eye(4, dtype=np.float32)
    shift[0, 3] = 5.0
    far = ctx.transform(s0, shift)
    prm = ctx.icp_params(max_correspondence_distance=0.05, max_iterations=30, transformation_epsilon=1e-8)
    g = np.stack([np.eye(4), S.turntable(12.0, S.OBJECT_AXIS), np.eye(4)]).astype(np.float32)
    res = ctx.icp_batch([s0, s0, far], [t0, t0, t0], prm, guesses=g)
    assert res[2].state == L.ICP_STATE_NO_CORRESPONDENCES and not res[2].converged
    assert res[0].status == L.NO_CORRESPONDENCES  # the call reports it
    _same(res[1], ctx.icp(s0, t0, prm, guess=g[1]))
    alone = ctx.icp(s0, t0, prm)
    np.testing.assert_array_equal(res[0].transform64, alone.transform64)


def test_empty_batch(ctx):
    assert ctx.icp_batch([], [], ctx.icp_params()) == []


def test_turntable_cycle_aligns_consecutive_views(ctx):
    caps, poses = S.turntable_cycle(seed=3, views=6, step_deg=10.0)
    p = ctx.depth_params(L.KINECT_V1, 640, 480, frames=1, scale=0.001, depth_max=4000.0, normals=False)
    cl = []
    for v in range(len(caps)):
        c = ctx.voxel_grid(ctx.backproject(caps[v], p), 0.001)
        cl.append(ctx.normals(c, 30))
    prm = ctx.icp_params(max_correspondence_distance=0.02, max_iterations=60, transformation_epsilon=1e-10,
                         euclidean_fitness_epsilon=1e-8, point_to_plane=True)
    # pair i: view i+1 onto view i; the ground truth maps view i+1's points to view i
    res = ctx.icp_batch(cl[1:], cl[:-1], prm)
    for i, r in enumerate(res):
        T_gt = poses[i] @ np.linalg.inv(poses[i + 1])
        xyz = xyz_of(cl[i + 1].download())
        assert r.converged
        assert S.rmse(r.transform64, T_gt, xyz) < 1e-3, (i, S.rmse(r.transform64, T_gt, xyz))


@pytest.mark.gpu
def test_stop_rule_ends_only_what_it_names(ctx, cfg0):
    """stop_iteration / stop_rms (no counterpart in PCL): a pair still above
    stop_rms after stop_iteration iterations ends there, not converged, with the
    transform of that iteration; a rule it never meets changes nothing."""
    s, t = ctx.upload(cfg0["vsrc"]), ctx.upload(cfg0["vtgt"])
    base = dict(max_correspondence_distance=0.05, max_iterations=50, transformation_epsilon=1e-8)
    free = ctx.icp(s, t, ctx.icp_params(**base))
    three = ctx.icp(s, t, ctx.icp_params(**{**base, "max_iterations": 3}))
    stopped = ctx.icp(s, t, ctx.icp_params(**base, stop_iteration=3, stop_rms=1e-9))
    assert stopped.state == L.ICP_STATE_STOPPED and not stopped.converged and stopped.iterations == 3
    np.testing.assert_array_equal(stopped.transform64, three.transform64)
    loose = ctx.icp(s, t, ctx.icp_params(**base, stop_iteration=3, stop_rms=1.0))
    np.testing.assert_array_equal(loose.transform64, free.transform64)
    assert loose.state == free.state and loose.iterations == free.iterations
    # in a batch each pair meets the rule on its own: a pair that stops leaves
    # the other's result as it is alone
    rule = ctx.icp_params(**base, stop_iteration=3, stop_rms=0.004)
    turned = ctx.upload(O.transform(cfg0["vsrc"], S.turntable(60.0, S.OBJECT_AXIS).astype(np.float32)))
    alone = [ctx.icp(a, t, rule) for a in (s, turned)]
    res = ctx.icp_batch([s, turned], [t, t], rule)
    for r, a in zip(res, alone):
        _same(r, a)
    assert any(r.state == L.ICP_STATE_STOPPED for r in res)
