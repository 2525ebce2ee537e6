"""Batched ragged clouds in one persistent launch: identical, bit for bit,
to one tree query per cloud, and to the oracle's exhaustive search."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def make_clouds(n_clouds, lo, hi, seed):
    from torch_kdtree_gb300.synthetic import ragged_clouds
    return ragged_clouds(n_clouds=n_clouds, lo=lo, hi=hi, seed=seed)


@pytest.mark.parametrize("tpq", [0, 8])
@pytest.mark.parametrize("boxes", [False, True])
def test_batch_matches_per_cloud_and_oracle(tpq, boxes, oracle):
    from torch_kdtree_gb300.batched import BatchedKDTrees
    clouds = make_clouds(24, 50, 20000, seed=3)
    refs = [torch.from_numpy(r).to(cuda) for r, _, _ in clouds]
    qs = [torch.from_numpy(q).to(cuda) for _, q, _ in clouds]
    ks = [k for _, _, k in clouds]
    b = BatchedKDTrees(refs, ks, [q.shape[0] for q in qs], threads_per_query=tpq, prune_boxes=boxes)
    d_b, i_b = b.query(qs)
    b.query_each(qs)
    d_e, i_e = b.split(b.out_dists), b.split(b.out_idx)
    for c, ((r, q, k), db, ib, de, ie) in enumerate(zip(clouds, d_b, i_b, d_e, i_e)):
        assert torch.equal(db, de) and torch.equal(ib, ie), c
        bd, bi = oracle.brute(r, q, k)
        np.testing.assert_array_equal(db.cpu().numpy(), bd)
        np.testing.assert_array_equal(ib.cpu().numpy(), bi)


def test_batch_graph_replay_and_large_k(oracle):
    from torch_kdtree_gb300.batched import BatchedKDTrees
    rng = np.random.default_rng(9)
    refs_np = [rng.standard_normal((n, 3)).astype(np.float32) for n in (300, 5000, 40000, 129)]
    qs_np = [rng.standard_normal((n, 3)).astype(np.float32) for n in (0, 2500, 7000, 64)]
    ks = [3, 100, 17, 128]
    b = BatchedKDTrees([torch.from_numpy(r).to(cuda) for r in refs_np], ks, [len(q) for q in qs_np],
                       levels=[2, None, 14, 1])
    q_flat = torch.from_numpy(np.concatenate(qs_np)).to(cuda)
    replay = b.graph(q_flat)
    b.out_dists.fill_(-1)
    replay()
    torch.cuda.synchronize()
    for (r, q, k, d, i) in zip(refs_np, qs_np, ks, b.split(b.out_dists), b.split(b.out_idx)):
        if len(q) == 0:
            continue
        bd, bi = oracle.brute(r, q, k)
        np.testing.assert_array_equal(d.cpu().numpy(), bd)
        np.testing.assert_array_equal(i.cpu().numpy(), bi)


def test_batch_errors():
    from torch_kdtree_gb300.batched import BatchedKDTrees
    r = torch.randn(10, 3, device=cuda)
    with pytest.raises(Exception):
        BatchedKDTrees([r], [11], [4])  # k > n
    with pytest.raises(Exception):
        BatchedKDTrees([r, torch.randn(10, 3, device=cuda, dtype=torch.float64)], [1, 1], [1, 1])
    b = BatchedKDTrees([r], [2], [4])
    with pytest.raises(Exception):
        b.query_flat(torch.randn(5, 3, device=cuda))  # wrong query count


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("dims", [4, 5, 6, 7, 8])
@pytest.mark.parametrize("tpq", [0, 1, 32])
def test_batch_of_wide_trees(dtype, dims, tpq, oracle):
    """Trees of 4-8 dimensions batched in one launch: the same bits as one
    query per cloud and as the oracle's exhaustive search, ties included."""
    from torch_kdtree_gb300.batched import BatchedKDTrees
    rng = np.random.default_rng(100 + dims)
    sizes = (40, 3000, 20000, 700, 9)
    refs_np = [rng.standard_normal((n, dims)).astype(dtype) for n in sizes]
    refs_np[1][:200] = refs_np[1][200:400]  # exact duplicates: ties
    qs_np = [rng.standard_normal((n, dims)).astype(dtype) for n in (30, 1200, 0, 500, 9)]
    ks = [5, 16, 1, 3, 9] if tpq == 1 else [5, 40, 1, 128, 9]
    levels = [None, 9, 11, None, 1]
    b = BatchedKDTrees([torch.from_numpy(r).to(cuda) for r in refs_np], ks, [len(q) for q in qs_np],
                       levels=levels, threads_per_query=tpq)
    qs = [torch.from_numpy(q).to(cuda) for q in qs_np]
    d_b, i_b = b.query(qs)
    b.query_each(qs)
    for c, (r, q, k, db, ib, de, ie) in enumerate(zip(refs_np, qs_np, ks, d_b, i_b, b.split(b.out_dists),
                                                      b.split(b.out_idx))):
        if len(q) == 0:
            continue
        assert torch.equal(db, de) and torch.equal(ib, ie), c
        bd, bi = oracle.brute(r, q, k)
        np.testing.assert_array_equal(db.cpu().numpy(), bd)
        np.testing.assert_array_equal(ib.cpu().numpy(), bi)


def test_random_batches(oracle):
    """A seeded sweep of batches: 1-12 clouds of one dims (1-8) and dtype,
    sizes from 2 up, per-cloud k and depth, empty query sets, every lane
    shape; each cloud's answer bit-exact against the exhaustive search."""
    from torch_kdtree_gb300.batched import BatchedKDTrees
    rng = np.random.default_rng(4242)
    for case in range(25):
        dims = int(rng.integers(1, 9))
        dtype = np.float32 if rng.random() < 0.75 else np.float64
        nc = int(rng.integers(1, 13))
        sizes = [int(rng.choice([2, 9, 150, 1200, 6000])) for _ in range(nc)]
        nqs = [int(rng.choice([0, 1, 33, 400])) for _ in range(nc)]
        tpq = int(rng.choice([0, 1, 8, 32]))
        kmax = 16 if tpq == 1 else 128
        ks = [int(rng.integers(1, min(n, kmax) + 1)) for n in sizes]
        levels = [int(rng.integers(1, int(np.log2(n)) + 1)) if rng.random() < 0.7 else None for n in sizes]
        refs_np = [rng.standard_normal((n, dims)).astype(dtype) for n in sizes]
        qs_np = [rng.standard_normal((m, dims)).astype(dtype) for m in nqs]
        if sum(nqs) == 0:
            continue
        b = BatchedKDTrees([torch.from_numpy(r).to(cuda) for r in refs_np], ks, nqs, levels=levels,
                           threads_per_query=tpq)
        d_b, i_b = b.query([torch.from_numpy(q).to(cuda) for q in qs_np])
        for c, (r, q, k, db, ib) in enumerate(zip(refs_np, qs_np, ks, d_b, i_b)):
            if len(q) == 0:
                continue
            bd, bi = oracle.brute(r, q, k)
            msg = f"case {case} cloud {c}: dims={dims} {np.dtype(dtype).name} n={len(r)} k={k} tpq={tpq}"
            np.testing.assert_array_equal(db.cpu().numpy(), bd, err_msg=msg)
            np.testing.assert_array_equal(ib.cpu().numpy(), bi, err_msg=msg)
