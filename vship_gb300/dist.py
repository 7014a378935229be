"""Host-side helpers for running one replica per GPU (frame pairs are independent, so nothing is
exchanged on the data path; ranks only agree on timing).

* ``max_over_ranks`` -- the slowest rank's time (the whole job ends when it does); works on the
  NCCL (device tensor) and gloo (host tensor) backends.
* ``shard_requests`` -- split a request stream over ranks by source, so that every request of a
  source lands on the same rank and its cached device state stays on one GPU; requests without a
  source key (never cached) go round-robin.
"""
from __future__ import annotations

import zlib


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_of_source(key: int, world: int) -> int:
    """Stable owner of a source key (same on every host and Python run)."""
    return zlib.crc32(int(key).to_bytes(8, "little")) % world


def shard_requests(requests, rank: int, world: int, key=lambda r: r[3]):
    """The requests of `requests` (in order) that rank `rank` of `world` serves."""
    out = []
    for i, r in enumerate(requests):
        k = key(r)
        owner = rank_of_source(k, world) if k else i % world
        if owner == rank:
            out.append(r)
    return out
