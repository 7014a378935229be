"""Replica helpers on two gloo ranks (CPU): the max over ranks, and a source-keyed request split
that covers the stream exactly once and keeps every source on one rank."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from vship_gb300 import dist as vd
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        m = vd.max_over_ranks(float(10 * rank + 3), world)
        stream = [(0.01 * i, i % 2, 1 + i % 16, (i * 7919) % 23 if i % 5 else 0, i % 8, [0]) for i in range(200)]
        mine = vd.shard_requests(stream, rank, world)
        objs = [None] * world
        dist.all_gather_object(objs, [stream.index(r) for r in mine])
        q.put((rank, m, objs))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    [p.start() for p in ps]
    res = [q.get(timeout=120) for _ in ps]
    [p.join(timeout=60) for p in ps]
    assert all(p.exitcode == 0 for p in ps)
    for rank, m, objs in res:
        assert m == 13.0
        a, b = set(objs[0]), set(objs[1])
        assert not (a & b) and a | b == set(range(200))
        stream = [(0.01 * i, i % 2, 1 + i % 16, (i * 7919) % 23 if i % 5 else 0, i % 8, [0]) for i in range(200)]
        for k in {r[3] for r in stream if r[3]}:
            owners = {0 if i in a else 1 for i, r in enumerate(stream) if r[3] == k}
            assert len(owners) == 1, k
