"""Replica sharding and the cross-rank combination of timings, on CPU with
two gloo ranks (the path itself has no exchange between GPUs)."""
from __future__ import annotations

import os
import socket

import pytest

from lowcost3dreconstruction_gb300.replicas import combine, shard


@pytest.mark.parametrize("weights,world", [([1.0] * 10, 2), ([5, 1, 1, 1, 1, 1], 2), ([3, 1, 4, 1, 5, 9, 2, 6], 3),
                                           ([1.0] * 3, 4), ([], 2), ([0, 0, 0, 0], 2)])
def test_shard_covers_every_item_once(weights, world):
    got = [list(shard(weights, r, world)) for r in range(world)]
    flat = [i for g in got for i in g]
    assert flat == list(range(len(weights)))
    if sum(weights) > 0 and len(weights) >= world:
        loads = [sum(weights[i] for i in g) for g in got]
        assert max(loads) <= sum(weights) / world + max(weights)


def test_shard_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard([1, 2], 2, 2)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        weights = [300, 280, 120, 90, 260, 250]
        mine = shard(weights, rank, world)
        # a rank's "time" grows with its work; counts are its aligned pairs
        t, c = combine(dist, [10.0 + rank, 1.0 * sum(weights[i] for i in mine)], [len(mine), 1.0])
        q.put((rank, list(mine), t, c))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_combine_max_time_and_summed_work():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    q = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    out.sort()
    ranges = [o[1] for o in out]
    assert sorted(ranges[0] + ranges[1]) == list(range(6))
    for _, _, t, c in out:
        assert t[0] == 11.0                      # slowest rank
        assert c == [6.0, 2.0]                   # every pair counted once; both ranks reported
    assert out[0][2] == out[1][2] and out[0][3] == out[1][3]
