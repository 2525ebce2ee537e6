"""Query sharding across processes, one GPU per process.

KNN queries are independent, so the path shards without any exchange: every
rank holds the same tree (built from the same cloud) and answers its own
contiguous range of the queries.  The only collectives are optional: gathering
the per-rank results into the full answer, and reducing per-rank timings.
Works with any torch.distributed backend (NCCL for CUDA tensors, gloo for CPU
tensors).

    start, stop = shard_range(len(q), rank, world)
    d, i = tree.query(q[start:stop], nr_nns_searches=k)
    d_all, i_all = gather_shards(d, i, len(q))       # optional
"""
from __future__ import annotations

from typing import Optional, Tuple

import torch


def shard_range(n: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous, balanced [start, stop) of n items for `rank` of `world`
    (sizes differ by at most one; every item belongs to exactly one rank)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} is not in a world of {world}")
    if n < 0:
        raise ValueError("n must be non-negative")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def world_max(value: float, device: Optional[torch.device] = None, group=None) -> float:
    """Maximum of a per-rank scalar over all ranks (the slowest rank's time);
    the value itself when torch.distributed is not initialised."""
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX, group=group)
    return float(t.item())


def gather_shards(dists: torch.Tensor, idx: torch.Tensor, n_total: int, group=None):
    """All-gather the per-rank results of a sharded query (rank r holding rows
    shard_range(n_total, r, world)) into the full [n_total, k] answer on every
    rank."""
    world = torch.distributed.get_world_size(group)
    rank = torch.distributed.get_rank(group)
    start, stop = shard_range(n_total, rank, world)
    if dists.shape[0] != stop - start or idx.shape[0] != stop - start:
        raise ValueError("local results do not match this rank's shard")
    k = dists.shape[1]
    rows = -(-n_total // world)  # the largest shard
    pad_d = dists.new_zeros((rows, k))
    pad_i = idx.new_full((rows, k), -1)
    pad_d[: stop - start] = dists
    pad_i[: stop - start] = idx
    all_d = [torch.empty_like(pad_d) for _ in range(world)]
    all_i = [torch.empty_like(pad_i) for _ in range(world)]
    torch.distributed.all_gather(all_d, pad_d, group=group)
    torch.distributed.all_gather(all_i, pad_i, group=group)
    out_d = dists.new_empty((n_total, k))
    out_i = idx.new_empty((n_total, k))
    for r in range(world):
        a, b = shard_range(n_total, r, world)
        out_d[a:b] = all_d[r][: b - a]
        out_i[a:b] = all_i[r][: b - a]
    return out_d, out_i
