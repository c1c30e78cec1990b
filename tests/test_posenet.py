"""Learned pose proposal.

CPU: the oracle's backward against finite differences of its own forward
(float64, no roundings), its pose <-> label conversions, and its sampler.
GPU: the sampler, the tensor-core encoder, the head and every gradient against
the oracle (bf16 roundings at the same points; the GPU accumulates in fp32 in
its own order, hence the tolerances written below), determinism, the
proposal's pose assembly, and that training lowers the loss."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import posenet as O


def random_pts(rng, clouds, n=O.PTS):
    """bf16-valued normalised clouds: noisy ellipsoid patches of different shapes."""
    out = np.zeros((clouds, n, 4), np.float32)
    for c in range(clouds):
        ax = rng.uniform(0.3, 1.0, 3)
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        p = u * ax + rng.normal(scale=0.02, size=(n, 3))
        out[c, :, :3] = O.bf16(p.astype(np.float32))
    return out


def random_params(rng, scale=1.0):
    p = np.zeros(O.PARAMS, np.float32)
    o = 0
    for name, shape in O.LAYOUT:
        k = int(np.prod(shape))
        if len(shape) == 2:
            a = np.sqrt(6.0 / shape[1]) * scale
            p[o:o + k] = rng.uniform(-a, a, k)
        else:
            p[o:o + k] = rng.normal(scale=0.1, size=k)
        o += k
    return p


# ------------------------------------------------------------------ CPU
def test_oracle_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    params = random_params(rng).astype(np.float64)
    pts = random_pts(rng, 4, n=48).astype(np.float64)
    labels = rng.normal(size=(2, 9))
    _, g, aux = O.loss_and_grads(params, pts, labels, exact=True)
    arg = aux["argmax"]
    eps = 1e-6
    o = 0
    for name, shape in O.LAYOUT:
        k = int(np.prod(shape))
        for j in rng.choice(k, size=min(k, 4), replace=False):
            i = o + int(j)
            pp, pm = params.copy(), params.copy()
            pp[i] += eps
            pm[i] -= eps
            lp = O.loss_and_grads(pp, pts, labels, argmax=arg, exact=True)[0]
            lm = O.loss_and_grads(pm, pts, labels, argmax=arg, exact=True)[0]
            fd = (lp - lm) / (2 * eps)
            assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (name, j, fd, g[i])
        o += k


def test_oracle_pose_label_round_trip():
    rng = np.random.default_rng(1)
    B = 5
    T = np.tile(np.eye(4), (B, 1, 1))
    for b in range(B):
        q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
        T[b, :3, :3] = q * np.sign(np.linalg.det(q))
        T[b, :3, 3] = rng.normal(scale=0.1, size=3)
    cs, ct = rng.normal(size=(B, 3)), rng.normal(size=(B, 3))
    lab = O.labels_from_transforms(T, cs, ct)
    np.testing.assert_allclose(O.transforms_from_outputs(lab, cs, ct), T, atol=1e-12)


def test_oracle_sample_is_stratified():
    idx = O.sample_indices(10_000, 7, 3)
    assert np.all(np.diff(idx) >= 0) and idx[0] >= 0 and idx[-1] < 10_000
    assert len(np.unique(idx)) > 0.99 * O.PTS   # adjacent strata may meet at their shared edge
    small = O.sample_indices(10, 7, 3)
    assert small.min() == 0 and small.max() == 9


# ------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def net(ctx):
    from lowcost3dreconstruction_gb300.posenet import PoseNet
    return PoseNet(ctx, seed=5)


def rel_err(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.gpu
def test_sample_matches_oracle(ctx, net):
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    rng = np.random.default_rng(2)
    xyz = [rng.normal(size=(n, 3)).astype(np.float32) * 0.1 + 1.0 for n in (5000, 777, 3)]
    xyz[1][5] = np.nan
    clouds = [ctx.upload(points_from_xyz(x)) for x in xyz]
    pts, cen = net.sample(clouds, seed=11)
    for c, x in enumerate(xyz):
        want, wc = O.sample(x, 11, c)
        np.testing.assert_allclose(cen[c], wc, rtol=0, atol=1e-12)
        # the centroids agree to FP64 summation order: at most one bf16 step apart
        np.testing.assert_allclose(pts[c], want, rtol=2 ** -7, atol=1e-6)


@pytest.mark.gpu
def test_encoder_and_head_forward_match_oracle(ctx, net):
    rng = np.random.default_rng(3)
    params = random_params(rng)
    net.set_params(params)
    pts = random_pts(rng, 6)
    feat, arg, y = net.forward(pts, train=True)
    f_ref, a_ref, y_ref, _ = O.forward(params, pts)
    # winners agree except where two points' channel values are within the fp32
    # accumulation difference of each other
    assert np.mean(arg == a_ref) > 0.99
    f_same, _, y_same, _ = O.forward(params, pts, argmax=arg)
    assert rel_err(feat, f_same) < 2e-3
    assert rel_err(feat, f_ref) < 2e-3
    assert rel_err(y, y_same) < 1e-2
    feat2, _, y2 = net.forward(pts, train=False)
    np.testing.assert_array_equal(feat2, feat)   # the inference kernel pools the same values
    np.testing.assert_array_equal(y2, y)


@pytest.mark.gpu
def test_gradients_match_oracle(ctx, net):
    rng = np.random.default_rng(4)
    params = random_params(rng)
    net.set_params(params)
    pts = random_pts(rng, 8)
    labels = rng.normal(size=(4, 9)).astype(np.float32)
    loss, g = net.gradients(pts, labels)
    _, arg, _ = net.forward(pts, train=True)
    l_ref, g_ref, _ = O.loss_and_grads(params, pts, labels, argmax=arg)
    # same winners, same bf16 roundings: what is left is fp32 summation order
    # (measured: loss 1.2e-4, every tensor <= 5.2e-4)
    assert abs(loss - l_ref) <= 1e-3 * abs(l_ref)
    G, R = O.split(g), O.split(g_ref)
    for name, _ in O.LAYOUT:
        assert rel_err(G[name], R[name]) < 1e-3, name
    loss2, g2 = net.gradients(pts, labels)
    assert loss2 == loss
    np.testing.assert_array_equal(g2, g)         # fixed summation orders: bit-reproducible


@pytest.mark.gpu
def test_propose_assembles_poses(ctx, net):
    """Output forced through the last bias: the guess must be
    Tr(c_tgt + delta/4) R Tr(-c_src) with R from Gram-Schmidt of the two columns."""
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    rng = np.random.default_rng(5)
    p = np.zeros(O.PARAMS, np.float32)
    ang = 0.7
    R = np.array([[np.cos(ang), 0, np.sin(ang)], [0, 1, 0], [-np.sin(ang), 0, np.cos(ang)]])
    delta = np.array([0.1, -0.2, 0.05])
    O.split(p)["c3"][:] = np.r_[R[:, 0] * 2.0, R[:, 1] + 0.3 * R[:, 0], delta]
    net.set_params(p)
    src = [ctx.upload(points_from_xyz(rng.normal(size=(3000, 3)) * 0.1)) for _ in range(2)]
    tgt = [ctx.upload(points_from_xyz(rng.normal(size=(2000, 3)) * 0.1 + 0.5)) for _ in range(2)]
    T = net.propose(src, tgt, seed=1)
    _, cen = net.sample(src + tgt, seed=1)
    for b in range(2):
        np.testing.assert_allclose(T[b, :3, :3], R, atol=1e-6)
        want_t = cen[2 + b] + delta / O.SCALE - R @ cen[b]
        np.testing.assert_allclose(T[b, :3, 3], want_t, atol=1e-6)


@pytest.mark.gpu
def test_training_lowers_the_loss(ctx):
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    from lowcost3dreconstruction_gb300.posenet import PoseNet, adamw
    rng = np.random.default_rng(6)
    n = PoseNet(ctx, seed=9)
    B = 8
    src, tgt, T = [], [], np.tile(np.eye(4, dtype=np.float32), (B, 1, 1))
    for b in range(B):
        xyz = rng.normal(size=(4000, 3)) * np.r_[0.15, 0.08, 0.04]
        a = rng.uniform(-np.pi, np.pi)
        R = np.array([[np.cos(a), 0, np.sin(a)], [0, 1, 0], [-np.sin(a), 0, np.cos(a)]])
        T[b, :3, :3] = R
        T[b, :3, 3] = rng.normal(scale=0.05, size=3)
        src.append(ctx.upload(points_from_xyz(xyz)))
        tgt.append(ctx.upload(points_from_xyz(xyz @ R.T + T[b, :3, 3])))
    losses = [n.train_step(src, tgt, T, seed=s, opt=adamw(lr=1e-3)) for s in range(30)]
    assert all(np.isfinite(losses))
    assert np.mean(losses[-5:]) < 0.5 * np.mean(losses[:3])


# ---------------------------------------------------- synthetic pairs, RMSE
@pytest.mark.gpu
def test_synthetic_pairs_are_seeded_rigid_and_visible(ctx):
    from lowcost3dreconstruction_gb300.core import xyz_of, normals_of
    s1, t1, T1 = ctx.synthetic_pairs(42, 3, 2000)
    s2, t2, T2 = ctx.synthetic_pairs(42, 3, 2000)
    np.testing.assert_array_equal(T1, T2)
    for a, b in zip(s1 + t1, s2 + t2):
        np.testing.assert_array_equal(a.download()["x"], b.download()["x"])
    for b in range(3):
        R = T1[b, :3, :3].astype(np.float64)
        np.testing.assert_allclose(R @ R.T, np.eye(3), atol=1e-5)
        assert np.linalg.det(R) > 0.999
        assert np.degrees(np.arccos(np.clip(R[1, 1], -1, 1))) <= 20.0 + 1e-3   # tilt bound
        assert np.all(np.abs(T1[b, :3, 3]) < 2.0)
        for c in (s1[b], t1[b]):
            p = c.download()
            xyz, nrm = xyz_of(p), normals_of(p)
            assert np.isfinite(xyz).all() and len(p) == 2000
            assert np.all(np.sum(nrm * xyz, axis=1) < 0)                     # every point faces the camera
            assert np.all(np.abs(np.linalg.norm(xyz, axis=1) - 1.0) < 0.6)   # about 1 m away
    # noise-free: the exact transform maps the source onto the target's surface
    s, t, T = ctx.synthetic_pairs(7, 2, 4000, yaw_deg=30, noise=False)
    for b in range(2):
        reg = ctx.transform(s[b], T[b])
        _, d = ctx.knn(t[b], reg, 1)
        assert np.median(np.sqrt(d[:, 0])) < 0.01


@pytest.mark.gpu
def test_rmse_batch_matches_numpy(ctx):
    from lowcost3dreconstruction_gb300.core import points_from_xyz
    rng = np.random.default_rng(8)
    xyz = [rng.normal(size=(n, 3)) for n in (1000, 37)]
    clouds = [ctx.upload(points_from_xyz(x)) for x in xyz]
    Ta = np.tile(np.eye(4), (2, 1, 1))
    Tb = Ta.copy()
    Tb[:, :3, 3] = [[0.001, 0, 0], [0, 0.002, 0.002]]
    Tb[1, :3, :3] = [[0, -1, 0], [1, 0, 0], [0, 0, 1]]
    got = ctx.rmse_batch(clouds, Ta, Tb)
    for i, x in enumerate(xyz):
        x32 = x.astype(np.float32).astype(np.float64)
        d = x32 @ (Ta[i, :3, :3] - Tb[i, :3, :3]).T + (Ta[i, :3, 3] - Tb[i, :3, 3])
        np.testing.assert_allclose(got[i], np.sqrt(np.mean(np.sum(d * d, axis=1))), rtol=1e-12)


# --------------------------------------------------------- trained network
@pytest.mark.gpu
def test_trained_proposal_gains_over_plain_icp(ctx):
    """The shipped network, on held-out pairs (seeds the training never drew):
    its proposals are within a few degrees, and proposal + ICP aligns more
    pairs per second than plain ICP from centroid alignment, with at least as
    many pairs aligned."""
    from lowcost3dreconstruction_gb300 import train_posenet as TP
    from lowcost3dreconstruction_gb300.posenet import WEIGHTS, PoseNet
    net = PoseNet(ctx)
    net.load(WEIGHTS)
    r = TP.evaluate(ctx, net, 200, seed=555_000_001, points=10000, chunk=200, yaw_deg=90.0)
    assert np.median(r.proposal_rot_err_deg) < 8.0
    assert np.mean(r.proposal_rot_err_deg < 30.0) > 0.9
    assert r.aligned_proposal >= r.aligned_plain
    assert r.pairs_per_s_proposal > 1.2 * r.pairs_per_s_plain


def test_oracle_reproduces_the_committed_fixture():
    """tests/golden/posenet_small.npz (tests/golden/make_golden.py posenet)
    pins the oracle's forward on seeded weights: winners exactly, values to
    FP32 rounding."""
    from pathlib import Path
    from oracle import posenet as OP
    g = np.load(Path(__file__).resolve().parent / "golden" / "posenet_small.npz")
    rng = np.random.default_rng(int(g["seed"]))
    params = (rng.standard_normal(OP.PARAMS) * 0.05).astype(np.float32)
    feat, argmax, y, _ = OP.forward(params, g["pts"])
    np.testing.assert_array_equal(argmax, g["argmax"])
    np.testing.assert_allclose(feat, g["feat"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(y, g["y"], rtol=1e-5, atol=1e-5)


@pytest.mark.gpu
def test_overlapped_fallback_equals_the_sequential_pipeline(ctx):
    """propose_refine with a second context (the fallback of the pairs the
    2 cm stage ended runs beside the 1 cm stage) gives every pair the result
    of the sequential order, field for field."""
    from lowcost3dreconstruction_gb300 import train_posenet as TP
    from lowcost3dreconstruction_gb300.core import Context
    from lowcost3dreconstruction_gb300.posenet import WEIGHTS, PoseNet
    net = PoseNet(ctx)
    net.load(WEIGHTS)
    srcs, tgts, _ = ctx.synthetic_pairs(424_242, 96, 8000, yaw_deg=180.0)
    # the sequential pipeline, written out
    seq = TP.refine(ctx, srcs, tgts, net.propose(srcs, tgts), TP.proposal_params())
    weak = [i for i, r in enumerate(seq) if not TP.settled(r)]
    fb = TP.refine(ctx, [srcs[i] for i in weak], [tgts[i] for i in weak],
                   TP.centroid_guesses(net, [srcs[i] for i in weak], [tgts[i] for i in weak]))
    for j, i in enumerate(weak):
        if TP.settled(fb[j]):
            seq[i] = fb[j]
    ctx2 = Context(0)
    try:
        for other in (None, ctx2):
            res, nfb = TP.propose_refine(ctx, net, srcs, tgts, other)
            assert nfb == len(weak) and nfb > 10
            for a, b in zip(res, seq):
                np.testing.assert_array_equal(a.transform64, b.transform64)
                assert (a.converged, a.iterations, a.state, a.n_correspondences, a.mse, a.fitness) == \
                    (b.converged, b.iterations, b.state, b.n_correspondences, b.mse, b.fitness)
    finally:
        ctx2.close()
