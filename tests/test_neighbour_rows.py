"""Neighbour rows (LCR_NORMALS_KEEP_NEIGHBOURS) and the correspondences ICP
proves from them.

NormalEstimation with keep_neighbours keeps each point's exact k nearest and
the largest squared distance R among them.  ICP then takes last iteration's
correspondence s of a source point q: when R > 4.0001 D(q, s), every target
point outside s's row is farther from q than s, so the capped nearest of q is
the nearest within the row -- no search.  The CPU test checks that claim on
adversarial clouds (lattices, duplicates) with distances rounded exactly as
FLANN's L2_Simple<float> does them; the GPU tests pin the rows to the oracle's
k-NN and ICP with rows to ICP without them, field for field.
"""
from __future__ import annotations

import numpy as np
import pytest

from lowcost3dreconstruction_gb300 import synthetic as S
from oracle import oracle as O


def _d2(q: np.ndarray, p: np.ndarray) -> np.ndarray:
    """Squared distances rounded like exact_dist2: float32 differences,
    squares, then ((d0 + d1) + d2)."""
    d = (q[:, None, :].astype(np.float32) - p[None, :, :].astype(np.float32)).astype(np.float32)
    s = (d * d).astype(np.float32)
    return ((s[..., 0] + s[..., 1]).astype(np.float32) + s[..., 2]).astype(np.float32)


def _nearest(D: np.ndarray, cols: np.ndarray | None = None):
    """(distance, index) minimum per row; cols restricts the candidates."""
    if cols is not None:
        D = np.where(cols, D, np.float32(np.inf))
    m = D.min(axis=1)
    idx = np.argmax(D == m[:, None], axis=1)  # lowest index among ties
    return m, idx


@pytest.mark.parametrize("kind", ["jitter", "lattice", "duplicates"])
def test_row_certificate_is_exact(kind):
    rng = np.random.default_rng({"jitter": 1, "lattice": 2, "duplicates": 3}[kind])
    g = np.stack(np.meshgrid(np.arange(40), np.arange(40), indexing="ij"), -1).reshape(-1, 2).astype(np.float64)
    pts = np.c_[g * 1e-3, np.zeros(len(g))] + np.array([0.3, -0.2, 1.1])
    if kind == "jitter":
        pts += rng.normal(scale=2e-4, size=pts.shape)
    if kind == "duplicates":
        pts = np.concatenate([pts, pts[rng.choice(len(pts), 300)]])
    pts = pts.astype(np.float32)
    k = 30
    Dpp = _d2(pts, pts)
    order = np.lexsort((np.broadcast_to(np.arange(len(pts)), Dpp.shape), Dpp), axis=1)[:, :k]
    R = np.take_along_axis(Dpp, order, axis=1).max(axis=1)
    # queries around the cloud, each with a seed among its few nearest
    q = (pts[rng.choice(len(pts), 1500)] + rng.normal(scale=1.5e-3, size=(1500, 3))).astype(np.float32)
    if kind == "lattice":  # exactly on lattice points and midpoints: distance ties
        q[:500] = pts[rng.choice(len(pts), 500)]
        q[500:800] = (pts[rng.choice(len(pts), 300)] + np.float32(5e-4)).astype(np.float32)
    Dq = _d2(q, pts)
    m_all, i_all = _nearest(Dq)
    rank = np.argsort(np.argsort(Dq, axis=1, kind="stable"), axis=1, kind="stable")
    s = np.array([rng.choice(np.flatnonzero(rank[j] < 6)) for j in range(len(q))])
    ds = Dq[np.arange(len(q)), s]
    ok = (R[s] > np.float32(4.0001) * ds) & (R[s] >= 1e-30) & ((ds == 0) | (ds >= 1e-30))
    assert ok.mean() > 0.5, ok.mean()
    member = np.zeros(Dq.shape, dtype=bool)
    np.put_along_axis(member, order[s], True, axis=1)
    m_row, i_row = _nearest(Dq, member)
    np.testing.assert_array_equal(m_row[ok].view(np.uint32), m_all[ok].view(np.uint32))
    np.testing.assert_array_equal(i_row[ok], i_all[ok])


def test_row_descent_is_exact():
    """The device's descent: from a far seed, hop to the row's nearest point
    while the test fails (at most 3 rows); a lane that passes at any hop gets
    its row's minimum, which must be the global nearest."""
    rng = np.random.default_rng(11)
    u = rng.uniform(-1, 1, size=(2500, 2))
    pts = np.c_[0.03 * u, 1.0 + 0.002 * np.sin(40 * u[:, 0])].astype(np.float32)
    pts = np.concatenate([pts, pts[:200]])  # duplicates
    k = 30
    Dpp = _d2(pts, pts)
    order = np.lexsort((np.broadcast_to(np.arange(len(pts)), Dpp.shape), Dpp), axis=1)[:, :k]
    R = np.take_along_axis(Dpp, order, axis=1).max(axis=1)
    q = (pts[rng.choice(len(pts), 1200)] + rng.normal(scale=[1e-3, 1e-3, 4e-4], size=(1200, 3))).astype(np.float32)
    Dq = _d2(q, pts)
    m_all, i_all = _nearest(Dq)
    rank = np.argsort(np.argsort(Dq, axis=1, kind="stable"), axis=1, kind="stable")
    proven = np.zeros(len(q), bool)
    hops = np.zeros(len(q), int)
    for j in range(len(q)):
        c = rng.choice(np.flatnonzero(rank[j] < 200))
        for hop in range(3):
            dc = Dq[j, c]
            row = order[c]
            d_row = Dq[j, row]
            m = d_row.min()
            b = row[d_row == m].min()
            if R[c] > np.float32(4.0001) * dc and R[c] >= 1e-30 and (dc == 0 or dc >= 1e-30):
                assert (m, b) == (m_all[j], i_all[j]), j
                proven[j] = True
                hops[j] = hop
                break
            if not (m < dc or (m == dc and b < c)):
                break
            c = b
    assert proven.mean() > 0.5 and (hops[proven] > 0).mean() > 0.2, (proven.mean(), (hops[proven] > 0).mean())


def _finite_cloud(seed: int, n: int) -> np.ndarray:
    """A wavy sheet of n points (x y z float32)."""
    rng = np.random.default_rng(seed)
    u = rng.uniform(-1, 1, size=(n, 2))
    return np.c_[0.2 * u, 1.0 + 0.05 * np.sin(6 * u[:, 0]) * np.cos(4 * u[:, 1])].astype(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("k", [30, 8])
def test_rows_hold_the_exact_k_nearest(ctx, k):
    rng = np.random.default_rng(5)
    xyz = _finite_cloud(5, 20000)
    xyz = np.concatenate([xyz, xyz[rng.choice(len(xyz), 500)]])  # duplicates
    xyz[rng.choice(len(xyz), 50)] = np.nan                      # non-finite points are skipped
    c = ctx.upload_xyz(xyz)
    plain = ctx.normals(c, k).download()
    kept = ctx.normals(c, k, keep_neighbours=True)
    # the normals themselves do not change
    got = kept.download()
    for f in plain.dtype.names:
        np.testing.assert_array_equal(got[f].view(np.uint32) if got[f].dtype.kind == "f" else got[f],
                                      plain[f].view(np.uint32) if plain[f].dtype.kind == "f" else plain[f])
    kk, rows = kept.neighbours()
    assert kk == k
    fin = np.all(np.isfinite(xyz), axis=1)
    oi, od = O.knn(got, got, k)
    for i in np.flatnonzero(fin):
        assert set(rows[i, :k].tolist()) == set(oi[i].tolist()), i
    np.testing.assert_array_equal(rows[fin, 31], od[fin, k - 1].view(np.uint32))


@pytest.mark.gpu
def test_rows_of_a_cloud_smaller_than_k(ctx):
    xyz = _finite_cloud(6, 12)
    kept = ctx.normals(ctx.upload_xyz(xyz), 30, keep_neighbours=True)
    k, rows = kept.neighbours()
    assert k == 30
    for i in range(12):
        assert sorted(rows[i, :12].tolist()) == list(range(12))
    assert np.all(rows[:, 31].view(np.float32) == np.inf)
    with pytest.raises(Exception):
        ctx.normals(ctx.upload_xyz(xyz), 30).neighbours()


def _same(a, b):
    np.testing.assert_array_equal(a.transform64, b.transform64)
    assert (a.converged, a.iterations, a.state, a.n_correspondences) == \
        (b.converged, b.iterations, b.state, b.n_correspondences)
    assert a.fitness == b.fitness and a.mse == b.mse


@pytest.fixture(scope="module")
def pairs(ctx):
    """Config-0 captures at three voxel sizes: sources, and targets with and
    without rows (the same normals)."""
    pr = S.config0_pair(0)
    prm = O.bp_params(640, 480, scale=0.001, depth_max=4000)
    src = O.backproject_v1(pr.src_frames[0], prm)
    tgt = O.backproject_v1(pr.tgt_frames[0], prm)
    out = []
    for leaf in (0.002, 0.003, 0.005):
        s, _ = O.voxel_grid(src, leaf)
        t, _ = O.voxel_grid(tgt, leaf)
        tc = ctx.upload(t)
        out.append((ctx.normals(ctx.upload(s), 30), ctx.normals(tc, 30), ctx.normals(tc, 30, keep_neighbours=True)))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("p2pl", [False, True])
@pytest.mark.parametrize("dist", [0.05, 0.005])
def test_icp_with_rows_equals_icp_without(ctx, pairs, p2pl, dist):
    """The 5 mm cap leaves many source tiles wider than four search radii
    (their unsettled lanes go one per warp; the settled ones leave results
    for the tile's row)."""
    prm = ctx.icp_params(max_correspondence_distance=dist, max_iterations=40, transformation_epsilon=1e-8,
                         point_to_plane=p2pl)
    g = np.stack([S.turntable(a, S.OBJECT_AXIS) for a in (0.0, 4.0, -6.0)]).astype(np.float32)
    without = ctx.icp_batch([s for s, _, _ in pairs], [t for _, t, _ in pairs], prm, guesses=g)
    with_rows = ctx.icp_batch([s for s, _, _ in pairs], [t for _, _, t in pairs], prm, guesses=g)
    assert max(r.iterations for r in without) > 3
    for a, b in zip(with_rows, without):
        _same(a, b)
    # a batch mixing targets with and without rows, and the single-pair call
    mixed = ctx.icp_batch([pairs[0][0], pairs[1][0]], [pairs[0][2], pairs[1][1]], prm, guesses=g[:2])
    _same(mixed[0], without[0])
    _same(mixed[1], without[1])
    _same(ctx.icp(pairs[2][0], pairs[2][2], prm, guess=g[2]), without[2])
