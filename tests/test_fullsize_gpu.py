"""Parity at the benchmark workloads' full sizes, against the oracle.

* differentiable KNN, 1,048,576 refs x 1,048,576 queries, k=8: forward vs
  the oracle's restatement of the reference CPU query on a sample; gradient
  vs the reference's torch-indexed formula (all rows) and vs FP64 central
  differences on a 4,096-query subset and reference points among their
  neighbours (neighbour lists held fixed);
* tensor-core brute force, 262,144 refs x 65,536 queries, d = 8 and 32, 5%
  duplicate refs, k=32: TF32 and BF16 hi/lo against the oracle's exhaustive
  search (the reference's distance arithmetic) on 1,024 queries;
* batched queries, the 256 ragged clouds: one graph replay of the batched
  launch against the oracle for 16 clouds (the largest, the smallest and
  every k).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def test_differentiable_workload_full_size():
    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300.synthetic import differentiable
    ref_np, q_np, w_np = differentiable()
    k = 8
    ref = torch.from_numpy(ref_np).to(cuda).requires_grad_(True)
    q = torch.from_numpy(q_np).to(cuda).requires_grad_(True)
    w = torch.from_numpy(w_np).to(cuda)
    dists, inds = tk.build_kd_tree(ref, levels=16).query(q, nr_nns_searches=k)
    (0.5 * (dists * w).sum()).backward()

    # forward: the oracle on a sample of queries (distances bitwise, indices up to exact ties)
    sample = 32768
    od, oi = O.query_tree(O.build_tree(ref_np), q_np[:sample], k)
    cmp = O.compare_knn(od, oi, dists[:sample].detach().cpu().numpy(), inds[:sample].cpu().numpy())
    assert cmp.ok, cmp

    # the reference's gradient: torch autograd through the re-gathered distances
    qq = q.detach().clone().requires_grad_(True)
    rr = ref.detach().clone().requires_grad_(True)
    dd = ((qq[:, None] - rr[inds.long()]) ** 2).sum(-1)
    (0.5 * (dd * w).sum()).backward()
    assert (q.grad - qq.grad).abs().max() <= 1e-5 * qq.grad.abs().max()
    assert (ref.grad - rr.grad).abs().max() <= 1e-5 * rr.grad.abs().max()

    # FP64 central differences with the neighbour lists held fixed
    h, m = 1e-4, 4096
    q64, r64, w64, il = q.detach().double(), ref.detach().double(), w.double(), inds.long()
    for c in range(3):
        e = torch.zeros(m, 3, dtype=torch.float64, device=cuda)
        e[:, c] = h
        lp = 0.5 * ((((q64[:m] + e)[:, None] - r64[il[:m]]) ** 2).sum(-1) * w64[:m]).sum(1)
        lm = 0.5 * ((((q64[:m] - e)[:, None] - r64[il[:m]]) ** 2).sum(-1) * w64[:m]).sum(1)
        fd = (lp - lm) / (2 * h)
        rel = ((q.grad[:m, c].double() - fd).abs() / fd.abs().clamp_min(1e-3)).max().item()
        assert rel < 1e-3, (c, rel)
    for mm in torch.unique(il[:m, 0])[:48].tolist():
        rows, cols = (il == mm).nonzero(as_tuple=True)
        for c in range(3):
            e = torch.zeros(3, dtype=torch.float64, device=cuda)
            e[c] = h

            def part(rv):
                return 0.5 * (((q64[rows] - rv) ** 2).sum(-1) * w64[rows, cols]).sum()

            fd = ((part(r64[mm] + e) - part(r64[mm] - e)) / (2 * h)).item()
            an = ref.grad[mm, c].item()
            assert abs(an - fd) <= 1e-3 * max(abs(fd), 1e-3), (mm, c, an, fd)


@pytest.mark.parametrize("d", [8, 32])
def test_tensor_core_brute_force_full_size(d):
    from torch_kdtree_gb300.nn_distance import nn_distance_raw
    from torch_kdtree_gb300.synthetic import tensor_core_brute
    ref_np, q_np = tensor_core_brute(d=d)
    k, sample = 32, 1024
    od, oi = O.brute(ref_np, q_np[:sample], k)
    ref = torch.from_numpy(ref_np).to(cuda)
    q = torch.from_numpy(q_np).to(cuda)
    for mode in ("tf32", "bf16_split", "exact"):
        dd = torch.empty(len(q), k, device=cuda)
        ii = torch.empty(len(q), k, dtype=torch.int32, device=cuda)
        nn_distance_raw(ref, q, k, dd, ii, mode)
        torch.cuda.synchronize()
        cmp = O.compare_knn(od, oi, dd[:sample].cpu().numpy(), ii[:sample].cpu().numpy())
        assert cmp.ok, (mode, cmp)
        # the oracle's exhaustive search breaks ties by lower index, as every mode does
        assert np.array_equal(oi, ii[:sample].cpu().numpy()), mode


def test_batched_ragged_clouds_full_size():
    from torch_kdtree_gb300.batched import BatchedKDTrees
    from torch_kdtree_gb300.synthetic import ragged_clouds
    clouds = ragged_clouds(n_clouds=256, seed=0)
    refs = [torch.from_numpy(r).to(cuda) for r, _, _ in clouds]
    qs = [torch.from_numpy(q).to(cuda) for _, q, _ in clouds]
    ks = [k for _, _, k in clouds]
    levels = [int(max(1, min(24, round(np.log2(max(2, len(r)) / 16))))) for r, _, _ in clouds]
    batch = BatchedKDTrees(refs, ks, [len(q) for q in qs], levels=levels)
    replay = batch.graph(torch.cat(qs).contiguous())
    batch.out_dists.zero_()
    batch.out_idx.fill_(-7)
    replay()
    torch.cuda.synchronize()
    sizes = np.array([len(r) for r, _, _ in clouds])
    order = np.argsort(sizes)
    pick = {int(order[0]), int(order[-1])}
    for kk in (1, 4, 16):
        with_k = [int(c) for c in order[::-1] if ks[c] == kk]
        pick.update(with_k[:: max(1, len(with_k) // 4)][:4])
    for c in order[:: max(1, len(order) // 16)]:
        if len(pick) >= 16:
            break
        pick.add(int(c))
    assert len(pick) >= 16 and {1, 4, 16} <= {ks[c] for c in pick}
    ds, is_ = batch.split(batch.out_dists), batch.split(batch.out_idx)
    for c in sorted(pick):
        r_np, q_np, kk = clouds[c]
        if len(r_np) * len(q_np) <= 2e8:
            od, oi = O.brute(r_np, q_np, kk)
        else:
            od, oi = O.query_tree(O.build_tree(r_np), q_np, kk)
        cmp = O.compare_knn(od, oi, ds[c].cpu().numpy(), is_[c].cpu().numpy())
        assert cmp.ok, (c, len(r_np), kk, cmp)
