"""The proposal pipeline's schedule on the host (no GPU): propose_refine, with
or without a second context for the early fallback, gives every pair the
result of the sequential order -- proposal, ICP at 2 cm then 1 cm, plain ICP
from the centroid guess for the pairs that did not settle.

A fake context stands in for the library.  Its ICP results depend only on the
pair, the stage's parameters and the starting transform, as a batched call's
do (each pair gets its single-pair result), so any schedule that runs the same
stages on the same pairs must produce the same results."""
from __future__ import annotations

import threading
import zlib

import numpy as np

from lowcost3dreconstruction_gb300 import _lib as L
from lowcost3dreconstruction_gb300 import train_posenet as TP


class FakeCloud:
    def __init__(self, i: int):
        self.i = i


class FakeResult:
    def __init__(self, state: int, converged: bool, mse: float, transform: np.ndarray):
        self.state, self.converged, self.mse, self.transform = state, converged, mse, transform

    def fields(self):
        return self.state, self.converged, self.mse, self.transform.tobytes()


class FakeContext:
    def __init__(self):
        self.calls = []
        self.lock = threading.Lock()

    def icp_batch(self, srcs, tgts, prm, guesses):
        with self.lock:
            self.calls.append((round(prm.max_correspondence_distance, 4), len(srcs)))
        out = []
        for s, t, g in zip(srcs, tgts, guesses):
            g = np.asarray(g, np.float32)
            key = f"{s.i}/{t.i}/{prm.max_correspondence_distance:.4f}".encode() + g.tobytes()
            rng = np.random.default_rng(zlib.crc32(key))
            state = int(rng.choice([L.ICP_STATE_TRANSFORM, L.ICP_STATE_ABS_MSE, L.ICP_STATE_STOPPED,
                                    L.ICP_STATE_NO_CORRESPONDENCES, L.ICP_STATE_ITERATIONS],
                                   p=[0.35, 0.15, 0.25, 0.1, 0.15]))
            converged = state in (L.ICP_STATE_TRANSFORM, L.ICP_STATE_ABS_MSE)
            mse = float(rng.uniform(0.0, 4e-5))
            T = (g + rng.normal(scale=1e-3, size=(4, 4))).astype(np.float32)
            out.append(FakeResult(state, converged, mse, T))
        return out


class FakeNet:
    def propose(self, srcs, tgts):
        return np.stack([np.eye(4, dtype=np.float32) * (1 + 1e-3 * s.i) for s in srcs])

    def sample(self, clouds):
        cen = np.array([[0.01 * c.i, -0.02 * c.i, 0.5] for c in clouds], np.float64)
        return None, cen


def _sequential(ctx, net, srcs, tgts):
    res = TP.refine(ctx, srcs, tgts, net.propose(srcs, tgts), TP.proposal_params())
    weak = [i for i, r in enumerate(res) if not TP.settled(r)]
    if weak:
        ws, wt = [srcs[i] for i in weak], [tgts[i] for i in weak]
        fb = TP.refine(ctx, ws, wt, TP.centroid_guesses(net, ws, wt))
        for j, i in enumerate(weak):
            if TP.settled(fb[j]):
                res[i] = fb[j]
    return res, len(weak)


def test_propose_refine_equals_the_sequential_order():
    n = 200
    srcs = [FakeCloud(2 * i) for i in range(n)]
    tgts = [FakeCloud(2 * i + 1) for i in range(n)]
    net = FakeNet()
    seq, nweak = _sequential(FakeContext(), net, srcs, tgts)
    assert 20 < nweak < n - 20
    ctx2 = FakeContext()
    for other in (None, ctx2):
        ctx = FakeContext()
        res, nfb = TP.propose_refine(ctx, net, srcs, tgts, other)
        assert nfb == nweak
        assert [r.fields() for r in res] == [r.fields() for r in seq]
    # with the second context, the fallback of the pairs the 2 cm stage ended
    # ran there (its 5 cm stage, then the 1 cm stage), and the fallback of the
    # pairs the 1 cm stage left unsettled ran on the first context after it
    assert ctx2.calls and ctx2.calls[0][0] == 0.05
    assert {c for c, _ in ctx2.calls} <= {0.05, 0.01}
    stages = [c for c, _ in ctx.calls]
    assert stages[:2] == [0.02, 0.01] and 0.05 in stages[2:]
