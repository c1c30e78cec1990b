"""Host-side logic of running the path as independent replicas, one process
per GPU: pairs are split into contiguous ranges balanced by their estimated
cost (no exchange inside a pair), and each step's clocks and counts are
combined across ranks -- the slowest rank's time, the sum of the work.  The
only collective is this one small all-reduce of timings; the data path has
none."""
from __future__ import annotations

from typing import Sequence


def shard(weights: Sequence[float], rank: int, world: int) -> range:
    """Contiguous range of item indices for `rank`: boundaries at the equal
    shares of the cumulative weight (each item goes to the rank whose share
    holds its midpoint), so every item is assigned exactly once."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world {world}")
    n = len(weights)
    total = float(sum(weights))
    if n == 0:
        return range(0, 0)
    if total <= 0:
        lo, hi = rank * n // world, (rank + 1) * n // world
        return range(lo, hi)
    cut = [0] * (world + 1)
    acc = 0.0
    r = 0
    for i, w in enumerate(weights):
        mid = acc + 0.5 * float(w)
        while r < world and mid >= total * (r + 1) / world:
            r += 1
            cut[r] = i
        acc += float(w)
    for k in range(r + 1, world + 1):
        cut[k] = n
    cut[world] = n
    return range(cut[rank], cut[rank + 1])


def combine(dist, times_ms: Sequence[float], counts: Sequence[float], device="cpu"):
    """All-reduce over the process group: max of each time, sum of each count.
    Returns (times, counts) as lists of floats, identical on every rank."""
    import torch
    t = torch.tensor(list(times_ms), dtype=torch.float64, device=device)
    c = torch.tensor(list(counts), dtype=torch.float64, device=device)
    if dist is not None and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.tolist()], [float(x) for x in c.tolist()]
