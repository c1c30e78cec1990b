"""The k-NN pass 1 histogram (search.cuh, KHist) modelled on the host: the
branchless form (every staged point adds 0 or 1 to its bin against the bound
at the start of the leaf, top bins dropped once per leaf) ends in the same
state as the per-candidate form (each candidate dropping bins as it arrives,
the bound shrinking within the leaf): the same boundary bin, and the same
counts in every bin below it, so pass 2 collects the same k-set.  When the
boundary is the open last bin, its count and its edge (its largest
candidate) may come out larger; the range still holds the keys pass 2
needs."""
from __future__ import annotations

import numpy as np
import pytest

BINS = 64


def _bits(d: np.float32) -> int:
    return int(np.float32(d).view(np.uint32))


class Hist:
    def __init__(self, K: int, top2: float, cap: float = np.inf):
        self.K, self.cap = K, np.float32(cap)
        self.e0 = (_bits(np.float32(top2)) >> 21) - (BINS - 1)
        self.h = np.zeros(BINS, np.int64)
        self.bs, self.cl, self.top_max = BINS, 0, np.float32(0.0)

    def bin(self, d) -> int:
        return min(max((_bits(d) >> 21) - self.e0, 0), BINS - 1)

    def edge(self, b: int) -> np.float32:
        top = b + self.e0 + 1
        if b >= BINS - 1:
            return self.top_max
        if top >= 1020:
            return np.float32(np.inf)
        return np.uint32((top << 21) - 1).view(np.float32)

    def bound(self) -> np.float32:
        return min(self.edge(self.bs - 1), self.cap) if self.cl >= self.K else self.cap

    def drop(self):
        while self.bs > 1:
            top = self.h[self.bs - 1]
            if self.cl - top < self.K:
                break
            self.cl -= top
            self.bs -= 1

    def leaf_per_candidate(self, ds):
        tau = self.bound()
        for d in ds:
            if not d <= tau:
                continue
            b = self.bin(d)
            if b == BINS - 1:
                self.top_max = max(self.top_max, d)
            self.h[b] += 1
            self.cl += 1
            if self.cl >= self.K:
                self.drop()
                tau = self.bound()

    def leaf_branchless(self, ds):
        tau = self.bound()
        for d in ds:
            c = bool(d <= tau)
            b = self.bin(d)
            self.h[b] += c
            if c and b == BINS - 1:
                self.top_max = max(self.top_max, d)
            self.cl += c
        if self.cl >= self.K:
            self.drop()


@pytest.mark.parametrize("case", range(60))
def test_branchless_pass1_ends_in_the_same_state(case):
    rng = np.random.default_rng(case)
    K = int(rng.choice([8, 30, 51]))
    nleaf = int(rng.integers(3, 25))
    scale = float(rng.choice([1e-6, 1e-3, 1.0]))
    ds = (rng.gamma(2.0, scale, size=(nleaf, 32)) ** 2).astype(np.float32)
    if case % 4 == 1:  # exact ties and duplicates
        ds = np.round(ds / (scale * scale) * 8) .astype(np.float32) * np.float32(scale * scale / 8)
    if case % 4 == 2:  # a range too low: neighbours pile into the open last bin
        top2 = float(np.percentile(ds, 2))
    elif case % 4 == 3:  # a range too high: everything clamps into bin 0
        top2 = float(ds.max()) * 1e12
    else:
        top2 = float(ds.max()) * 4
    if case % 5 == 0:
        ds[0, :5] = 0.0  # the query itself and duplicates of it
    a, b = Hist(K, top2), Hist(K, top2)
    for leaf in ds:
        a.leaf_per_candidate(leaf)
        b.leaf_branchless(leaf)
    # the same boundary bin and the same counts below it; the boundary's own
    # count agrees too unless it is the open last bin
    assert a.bs == b.bs
    bb = a.bs - 1
    np.testing.assert_array_equal(a.h[:bb], b.h[:bb])
    if bb < BINS - 1:
        assert a.h[bb] == b.h[bb] and a.cl == b.cl and a.bound() == b.bound()
    else:
        assert b.top_max >= a.top_max
    # pass 2: every key below the boundary bin, and the m smallest keys of the
    # boundary range, are the K nearest under the (distance, index) order
    keys = sorted((float(d), i) for i, d in enumerate(ds.ravel()))
    want = set(keys[:K])
    for h in (a, b):
        assert h.cl >= K
        lo = h.edge(bb - 1) if bb > 0 else -np.inf
        hi = h.edge(bb)
        below = [k for k in keys if k[0] <= lo]
        boundary = [k for k in keys if lo < k[0] <= hi]
        m = K - len(below)
        assert len(below) == h.cl - h.h[bb] and 0 < m <= len(boundary)
        assert set(below) | set(boundary[:m]) == want
