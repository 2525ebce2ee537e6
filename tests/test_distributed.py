"""Sharded queries across processes (torch_kdtree_gb300.distributed), on CPU
with the gloo backend and world size 2: the shards cover every query once,
the gathered answer equals one process's exhaustive answer, and timings
reduce to the slowest rank.  Each rank computes its shard with the oracle
(this host logic is the same whichever device answers the shard)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp


def test_shard_range_covers_everything_once():
    from torch_kdtree_gb300.distributed import shard_range
    for n in (0, 1, 7, 1000, 1001, 1 << 20):
        for world in (1, 2, 3, 8):
            owner = np.zeros(n, np.int64)
            sizes = []
            for r in range(world):
                a, b = shard_range(n, r, world)
                owner[a:b] += 1
                sizes.append(b - a)
            assert (owner == 1).all()
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, ref, q, k, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        from torch_kdtree_gb300.distributed import gather_shards, shard_range, world_max
        a, b = shard_range(len(q), rank, world)
        d, i = O.brute(ref, q[a:b], k, nthreads=2)
        dd, ii = gather_shards(torch.from_numpy(d), torch.from_numpy(i), len(q))
        t = world_max(float(10 * (rank + 1)))
        np.savez(f"{out_path}.{rank}.npz", d=dd.numpy(), i=ii.numpy(), t=t)
    finally:
        torch.distributed.destroy_process_group()


def test_two_ranks_gloo(tmp_path, oracle):
    rng = np.random.default_rng(7)
    ref = rng.standard_normal((3000, 3)).astype(np.float32)
    q = rng.standard_normal((1001, 3)).astype(np.float32)  # uneven split
    k = 4
    out = str(tmp_path / "res")
    mp.spawn(_worker, args=(2, _free_port(), ref, q, k, out), nprocs=2, join=True)
    bd, bi = oracle.brute(ref, q, k)
    for r in range(2):
        z = np.load(f"{out}.{r}.npz")
        np.testing.assert_array_equal(z["d"], bd)
        np.testing.assert_array_equal(z["i"], bi)
        assert float(z["t"]) == 20.0
