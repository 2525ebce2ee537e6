"""CPU trees (build_kd_tree(..., device='cpu')), the reference's KDTreeCPU
path (torch_kdtree/nn_distance.py:23-26, src/interface.cpp:128-141):
built and queried on the host by the library's own threaded search
(tk_tree_query_cpu).  Checked against the oracle's exhaustive search (same
contract: reference arithmetic, lower index among ties) bit for bit, and
against the reference's own outputs (golden fixtures) up to exact ties.
Runs without a GPU."""
import numpy as np
import pytest
import torch

from golden_util import inputs_of, rows
from make_golden import CASES

NAMES = [c[0] for c in CASES]


def tk():
    import torch_kdtree_gb300
    return torch_kdtree_gb300


@pytest.mark.parametrize("name", NAMES)
def test_cpu_tree_matches_oracle_and_reference(name, oracle, golden):
    case = golden[name]
    ref, q = inputs_of(case)
    k = int(case["k"])
    tree = tk().build_kd_tree(torch.from_numpy(ref), device="cpu", levels=int(case["levels"]))
    assert tree.built_on == "host" and not tree.use_gpu
    d, i = tree.query(torch.from_numpy(q), nr_nns_searches=k)
    assert d.device.type == "cpu" and i.dtype == torch.int32
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(d.numpy(), bd)
    np.testing.assert_array_equal(i.numpy(), bi)
    r = rows(case)
    cmp = oracle.compare_knn(case["dists"], case["idx"], d.numpy()[:r], i.numpy()[:r])
    assert cmp.ok, cmp


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3, 4, 6, 8])
def test_cpu_tree_every_depth_and_large_k(dtype, d, oracle):
    rng = np.random.default_rng(d)
    ref = rng.standard_normal((3000, d)).astype(dtype)
    ref[100:200] = ref[:100]  # exact duplicates: ties
    q = rng.standard_normal((400, d)).astype(dtype)
    q[:20] = ref[300:320]     # queries on reference points: zero distances
    for levels in (1, 4, 8):
        for k in (1, 7, 200):
            tree = tk().build_kd_tree(torch.from_numpy(ref), device="cpu", levels=levels)
            dd, ii = tree.query(torch.from_numpy(q), nr_nns_searches=k)
            bd, bi = oracle.brute(ref, q, k)
            np.testing.assert_array_equal(dd.numpy(), bd)
            np.testing.assert_array_equal(ii.numpy(), bi)


def test_cpu_tree_k_equal_to_n_and_nan_rows(oracle):
    rng = np.random.default_rng(3)
    ref = rng.standard_normal((30, 3)).astype(np.float32)
    q = rng.standard_normal((12, 3)).astype(np.float32)
    q[5, 1] = np.nan
    tree = tk().build_kd_tree(torch.from_numpy(ref), device="cpu")
    d, i = tree.query(torch.from_numpy(q), nr_nns_searches=30)
    assert torch.isinf(d[5]).all() and (i[5] == -1).all()
    keep = np.r_[0:5, 6:12]
    bd, bi = oracle.brute(ref, q[keep], 30)
    np.testing.assert_array_equal(d.numpy()[keep], bd)
    np.testing.assert_array_equal(i.numpy()[keep], bi)
    assert sorted(i[0].tolist()) == list(range(30))


def test_cpu_tree_api_surface(tmp_path, oracle):
    rng = np.random.default_rng(4)
    ref = torch.from_numpy(rng.standard_normal((5000, 3)).astype(np.float32))
    q = torch.from_numpy(rng.standard_normal((300, 3)).astype(np.float32))
    tree = tk().build_kd_tree(ref, device="cpu", squared_distances=False)
    d, i = tree.query(q, nr_nns_searches=6)
    bd, bi = oracle.brute(ref.numpy(), q.numpy(), 6)
    assert torch.equal(d, torch.sqrt(torch.from_numpy(bd)))  # the reference applies torch.sqrt
    # caller buffers
    rd = torch.empty(300, 6)
    ri = torch.empty(300, 6, dtype=torch.int32)
    tree2 = tk().build_kd_tree(ref, device="cpu")
    d2, i2 = tree2.query(q, nr_nns_searches=6, result_dists=rd, result_idx=ri)
    assert d2.data_ptr() == rd.data_ptr() and i2.data_ptr() == ri.data_ptr()
    np.testing.assert_array_equal(rd.numpy(), bd)
    # the layout the reference exposes
    assert tree2.structured_points.shape == (5000, 3) and tree2.shuffled_ind.dtype == torch.int64
    np.testing.assert_array_equal(tree2.structured_points.numpy(), ref.numpy()[tree2.shuffled_ind.numpy()])
    # save / load onto the CPU
    p = tmp_path / "t.npz"
    tree2.save(p)
    t3 = tk().load_kd_tree(p, device="cpu")
    d3, i3 = t3.query(q, nr_nns_searches=6)
    assert torch.equal(d3, rd) and torch.equal(i3, ri)
    # errors as the reference raises them
    with pytest.raises(RuntimeError):
        tree2.query(q, nr_nns_searches=5001)
    with pytest.raises(AssertionError):
        tree2.query(q.double(), nr_nns_searches=2)


def test_cpu_tree_gradient_is_the_reference_formula():
    rng = np.random.default_rng(5)
    ref = torch.from_numpy(rng.standard_normal((2000, 3))).requires_grad_(True)
    q = torch.from_numpy(rng.standard_normal((500, 3))).requires_grad_(True)
    w = torch.rand(500, 4, dtype=torch.float64)
    d, i = tk().build_kd_tree(ref, device="cpu").query(q, nr_nns_searches=4)
    (0.5 * (d * w).sum()).backward()
    il = i.long()
    gq = (w[..., None] * (q.detach()[:, None] - ref.detach()[il])).sum(1)
    assert torch.allclose(q.grad, gq, rtol=1e-12, atol=1e-12)
    gr = torch.zeros_like(ref).index_add_(0, il.reshape(-1), (-w[..., None] * (q.detach()[:, None] -
                                                                              ref.detach()[il])).reshape(-1, 3))
    assert torch.allclose(ref.grad, gr, rtol=1e-10, atol=1e-12)


def test_cpu_query_rejects_a_null_tree():
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL
    d = np.empty((1, 1), np.float32)
    i = np.empty((1, 1), np.int32)
    q = np.zeros((1, 3), np.float32)
    assert LIB.tk_tree_query_cpu(None, q.ctypes.data, 1, 1, d.ctypes.data, i.ctypes.data, 0) == TK_EINVAL
    assert b"null" in LIB.tk_last_error()


def test_cpu_query_order_and_threads_do_not_change_answers(oracle):
    """The host search takes queries in tree-cell order (from 128 queries on)
    in 256-query chunks pulled by the threads: every batch size around those
    boundaries and every thread count gives the exhaustive search's answer."""
    import ctypes
    from torch_kdtree_gb300._lib import LIB
    rng = np.random.default_rng(11)
    ref = rng.standard_normal((2000, 3)).astype(np.float32)
    ref[50:80] = ref[:30]  # exact duplicates: ties
    q_all = (rng.standard_normal((4099, 3)) * 1.3).astype(np.float32)
    k = 9
    tree = tk().build_kd_tree(torch.from_numpy(ref), device="cpu", levels=6)
    h = tree._tree.handle
    for nq in (1, 63, 127, 128, 129, 255, 257, 1000, 4099):
        q = np.ascontiguousarray(q_all[:nq])
        bd, bi = oracle.brute(ref, q, k)
        for threads in (1, 3, 16):
            d = np.empty((nq, k), np.float32)
            i = np.empty((nq, k), np.int32)
            assert LIB.tk_tree_query_cpu(h, q.ctypes.data, nq, k, d.ctypes.data, i.ctypes.data, threads) == 0
            np.testing.assert_array_equal(d, bd, err_msg=f"nq={nq} threads={threads}")
            np.testing.assert_array_equal(i, bi, err_msg=f"nq={nq} threads={threads}")
