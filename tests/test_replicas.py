"""Multi-rank host logic on CPU (gloo, world size 2): work sharding and the
max / sum reductions bench.py uses for the slowest-rank step time."""

from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, world: int, port: int, out) -> None:
    import torch.distributed as dist

    from pyloki_gb300.replicas import max_over_ranks, shard, sum_over_ranks

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard(list(range(7)), rank, world)
        slow = max_over_ranks(10.0 + rank * 5.0, dist)
        total = sum_over_ranks(len(mine), dist)
        out.put((rank, mine, slow, total))
    finally:
        dist.destroy_process_group()


def test_shard_covers_every_item_once():
    from pyloki_gb300.replicas import shard

    items = list(range(11))
    parts = [shard(items, r, 3) for r in range(3)]
    assert sorted(x for p in parts for x in p) == items
    assert max(map(len, parts)) - min(map(len, parts)) <= 1
    with pytest.raises(ValueError):
        shard(items, 3, 3)


def test_two_gloo_ranks_agree_on_slowest_and_total():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [[0, 2, 4, 6], [1, 3, 5]]
    assert all(r[2] == 15.0 for r in res)  # max over ranks
    assert all(r[3] == 7.0 for r in res)   # every item processed once


def test_single_process_reductions_are_identity():
    from pyloki_gb300.replicas import max_over_ranks, sum_over_ranks

    assert max_over_ranks(3.5) == 3.5
    assert sum_over_ranks(4) == 4.0
