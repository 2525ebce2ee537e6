"""GPU parity of the KD-tree query (through the C ABI via the Python API).

Bar: bit-exact against the oracle's exhaustive search ordered by
(distance, original index); against the reference's own outputs (golden
fixtures), distances bitwise and indices equal except inside exact ties."""
import numpy as np
import pytest
import torch

from golden_util import inputs_of, rows
from make_golden import CASES

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def tk():
    import torch_kdtree_gb300
    return torch_kdtree_gb300


def gpu_query(ref, q, k, levels=None, **opts):
    from torch_kdtree_gb300._lib import QueryOpts
    qo = QueryOpts.make(**opts) if opts else None
    tree = tk().build_kd_tree(torch.from_numpy(ref).to(cuda), levels=levels, query_opts=qo)
    d, i = tree.query(torch.from_numpy(q).to(cuda), nr_nns_searches=k)
    torch.cuda.synchronize()
    return d.cpu().numpy(), i.cpu().numpy()


@pytest.mark.parametrize("name", [c[0] for c in CASES])
def test_golden_fixtures(name, golden, oracle):
    case = golden[name]
    ref, q = inputs_of(case)
    k = int(case["k"])
    d, i = gpu_query(ref, q, k, levels=int(case["levels"]))
    # canonical answer: bit-exact
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(d, bd)
    np.testing.assert_array_equal(i, bi)
    # the reference's own answer: equal up to exact-distance ties
    r = rows(case)
    cmp = oracle.compare_knn(case["dists"], case["idx"], d[:r], i[:r])
    assert cmp.ok, cmp


@pytest.mark.parametrize("tpq", [1, 2, 4, 8, 16, 32])
@pytest.mark.parametrize("k", [1, 5, 16, 33, 128])
def test_launch_shapes_give_identical_results(tpq, k, oracle):
    rng = np.random.default_rng(11)
    ref = rng.standard_normal((20000, 3)).astype(np.float32)
    q = (rng.standard_normal((3000, 3)) * 1.2).astype(np.float32)
    bd, bi = oracle.brute(ref, q, k)
    for binq in (0, 1):
        for boxes in (0, 1):
            d, i = gpu_query(ref, q, k, levels=9, threads_per_query=tpq, bin_queries=binq, prune_boxes=boxes)
            np.testing.assert_array_equal(d, bd)
            np.testing.assert_array_equal(i, bi)


@pytest.mark.parametrize("levels", [1, 2, 3, 7, 11, 13, 14])
def test_any_tree_depth_gives_identical_results(levels, oracle):
    rng = np.random.default_rng(12)
    ref = rng.random((20000, 3)).astype(np.float32)
    q = (rng.random((2500, 3)) * 1.2 - 0.1).astype(np.float32)
    bd, bi = oracle.brute(ref, q, 16)
    for smem in (0, 5, 12):
        for boxes, trav in ((0, 1), (1, 1), (1, 2)):
            d, i = gpu_query(ref, q, 16, levels=levels, smem_levels=smem, prune_boxes=boxes, traversal=trav)
            np.testing.assert_array_equal(d, bd)
            np.testing.assert_array_equal(i, bi)


@pytest.mark.parametrize("k", [1, 2, 3, 5, 8, 13, 16, 17, 64])
@pytest.mark.parametrize("levels", [4, 9, 12])
def test_warp_packets_give_identical_results(k, levels, oracle):
    """Warp-packet traversal (one lane per query, the warp walks the tree
    together): exact for every k it serves, query counts that leave warps
    partly empty, unbinned order, and k > 16 (falls back to per-query)."""
    rng = np.random.default_rng(16)
    ref = rng.standard_normal((30000, 3)).astype(np.float32)
    q = (rng.standard_normal((3001, 3)) * 1.3).astype(np.float32)
    bd, bi = oracle.brute(ref, q, k)
    for binq in (0, 1):
        d, i = gpu_query(ref, q, k, levels=levels, traversal=2, bin_queries=binq)
        np.testing.assert_array_equal(d, bd)
        np.testing.assert_array_equal(i, bi)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_warp_packets_all_instantiations(dtype, d, oracle):
    rng = np.random.default_rng(17 + d)
    ref = (rng.standard_normal((5000, d)) * 1e3).astype(dtype)
    q = (rng.standard_normal((777, d)) * 1e3).astype(dtype)
    # a cloud with heavy exact duplicates (ties across leaves)
    ref[2500:] = ref[:2500]
    for k in (1, 4, 16):
        bd, bi = oracle.brute(ref, q, k)
        d_, i_ = gpu_query(ref, q, k, levels=8, traversal=2)
        np.testing.assert_array_equal(d_, bd)
        np.testing.assert_array_equal(i_, bi)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_reference_test_grid(dtype, d, oracle):
    """The grid of the reference's test_kdtree (tests/test_knn_unit.py:30-70):
    refs x queries x k, N(0,1)*1e3 data, k > N must raise."""
    rng = np.random.default_rng(100 + d)
    for nr_refs in (5, 10, 20, 30, 1000, 10000):
        ref = (rng.standard_normal((nr_refs, d)) * 1e3).astype(dtype)
        tree = tk().build_kd_tree(torch.from_numpy(ref).to(cuda))
        for nr_query in (5, 10, 20, 30, 1000):
            q = (rng.standard_normal((nr_query, d)) * 1e3).astype(dtype)
            qt = torch.from_numpy(q).to(cuda)
            for k in (1, 5, 10, 20):
                if k > nr_refs:
                    with pytest.raises(Exception):
                        tree.query(qt, nr_nns_searches=k)
                    continue
                dists, inds = tree.query(qt, nr_nns_searches=k)
                assert dists.device.type == "cuda" and inds.device.type == "cuda"
                assert inds.shape == (nr_query, k) and dists.shape == (nr_query, k)
                bd, bi = oracle.brute(ref, q, k)
                np.testing.assert_array_equal(dists.cpu().numpy(), bd)
                np.testing.assert_array_equal(inds.cpu().numpy(), bi)


def test_duplicate_points_ties_break_by_lower_index(oracle):
    rng = np.random.default_rng(13)
    base = rng.standard_normal((500, 3)).astype(np.float32)
    ref = np.concatenate([base, base, base[:100]])  # exact duplicates, later copies have higher indices
    q = base[:200] + np.float32(1e-3)
    d, i = gpu_query(ref, q, 6)
    bd, bi = oracle.brute(ref, q, 6)
    np.testing.assert_array_equal(i, bi)
    np.testing.assert_array_equal(d, bd)
    # each query sees its source point twice (or three times) at equal distance: lower index first
    assert np.all(i[:, 0] < i[:, 1])


def test_api_errors():
    t = tk()
    pts = torch.randn(10, 3, device=cuda)
    tree = t.build_kd_tree(pts)
    with pytest.raises(Exception):
        tree.query(torch.randn(10, 3, dtype=torch.float64, device=cuda))  # wrong dtype
    with pytest.raises(Exception):
        tree.query(torch.randn(5, 3, device=cuda), nr_nns_searches=11)  # k > N
    with pytest.raises(Exception):
        t.build_kd_tree(np.random.uniform(size=(10, 436)), device="cuda")  # uncompiled dimension
    with pytest.raises(Exception):
        t.build_kd_tree(torch.randn(10, 3), device="meta")  # trees live on a CUDA device or the CPU
    from torch_kdtree_gb300._lib import QueryOpts
    bad = t.build_kd_tree(pts, query_opts=QueryOpts.make(traversal=3))
    with pytest.raises(Exception):
        bad.query(torch.randn(5, 3, device=cuda))  # unknown traversal


def test_empty_query_and_result_buffers(oracle):
    rng = np.random.default_rng(14)
    ref = rng.standard_normal((1000, 3)).astype(np.float32)
    tree = tk().build_kd_tree(torch.from_numpy(ref).to(cuda))
    d, i = tree.query(torch.empty(0, 3, device=cuda), nr_nns_searches=4)
    assert d.shape == (0, 4) and i.shape == (0, 4)
    q = rng.standard_normal((64, 3)).astype(np.float32)
    rd = torch.empty(64, 4, device=cuda)
    ri = torch.empty(64, 4, dtype=torch.int32, device=cuda)
    d, i = tree.query(torch.from_numpy(q), nr_nns_searches=4, result_dists=rd, result_idx=ri)  # host query
    assert d.data_ptr() == rd.data_ptr() and i.data_ptr() == ri.data_ptr()
    bd, bi = oracle.brute(ref, q, 4)
    np.testing.assert_array_equal(rd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ri.cpu().numpy(), bi)


def test_sqrt_distances():
    pts = torch.randn(2000, 3, device=cuda)
    q = torch.randn(100, 3, device=cuda)
    d2, i2 = tk().build_kd_tree(pts).query(q, nr_nns_searches=3)
    d1, i1 = tk().build_kd_tree(pts, squared_distances=False).query(q, nr_nns_searches=3)
    assert torch.equal(i1, i2)
    assert torch.equal(d1, torch.sqrt(d2))


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_grad_like_reference(dtype):
    """tests/test_knn_unit.py:90-107 of the reference."""
    dims = 3
    points_ref = torch.randn(size=(10, dims), dtype=dtype, device=cuda, requires_grad=True)
    t_kdtree = tk().build_kd_tree(points_ref)
    points_query = torch.randn(size=(5, dims), dtype=dtype, device=cuda, requires_grad=True)
    dists, inds = t_kdtree.query(points_query, nr_nns_searches=2)
    (0.5 * torch.sum(dists)).backward()
    assert points_query.grad is not None
    assert torch.allclose(points_query.grad, torch.sum((points_query[:, None] - points_ref[inds.long()]), axis=-2))
    assert points_ref.grad is not None
    points_ref_grad = torch.zeros_like(points_ref)
    for i, ind in enumerate(inds.long()):
        points_ref_grad[ind] += points_ref[ind] - points_query[i]
    assert torch.allclose(points_ref.grad, points_ref_grad)


def test_nan_query_row_is_isolated(oracle):
    rng = np.random.default_rng(15)
    ref = rng.standard_normal((5000, 3)).astype(np.float32)
    q = rng.standard_normal((300, 3)).astype(np.float32)
    q[17, 1] = np.nan
    d, i = gpu_query(ref, q, 4)
    ok = np.ones(300, bool)
    ok[17] = False
    bd, bi = oracle.brute(ref, q[ok], 4)
    np.testing.assert_array_equal(d[ok], bd)
    np.testing.assert_array_equal(i[ok], bi)


WIDE_FIXTURES = ["wide_f32_d4_n1000_q200_k10", "wide_f32_d5_n10000_q300_k20", "wide_f32_d8_n10000_q300_k16",
                 "wide_f64_d6_n1000_q200_k10", "wide_f64_d8_n5000_q200_k33", "wide_f32_d7_n30_q20_k5",
                 "wide_ties_f32_d4_grid"]


@pytest.mark.parametrize("name", WIDE_FIXTURES)
def test_wide_golden_fixtures(name, golden, oracle):
    """Trees of 4-8 dimensions (the reference's README recipe) against the
    reference's own outputs and the oracle's exhaustive answer."""
    case = golden[name]
    ref, q = inputs_of(case)
    k = int(case["k"])
    d, i = gpu_query(ref, q, k, levels=int(case["levels"]))
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(d, bd)
    np.testing.assert_array_equal(i, bi)
    r = rows(case)
    cmp = oracle.compare_knn(case["dists"], case["idx"], d[:r], i[:r])
    assert cmp.ok, cmp


@pytest.mark.parametrize("dims", [4, 5, 6, 7, 8])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_wide_trees_every_shape(dims, dtype, oracle):
    rng = np.random.default_rng(60 + dims)
    ref = rng.standard_normal((6000, dims)).astype(dtype)
    q = (rng.standard_normal((1500, dims)) * 1.2).astype(dtype)
    for k in (1, 5, 16, 17, 100):
        bd, bi = oracle.brute(ref, q, k)
        for levels in (1, 5, 9):
            # binq=1 forces the cell + cost-class launch order on this small batch
            for tpq, boxes, binq in ((0, 1, -1), (1, 1, 1), (1, 0, -1), (32, 1, 1), (8, 0, -1), (32, 0, 1)):
                d, i = gpu_query(ref, q, k, levels=levels, threads_per_query=tpq, prune_boxes=boxes, bin_queries=binq)
                np.testing.assert_array_equal(d, bd, err_msg=f"k={k} L={levels} tpq={tpq} boxes={boxes} binq={binq}")
                np.testing.assert_array_equal(i, bi)


def test_wide_tree_build_save_load_and_grad(tmp_path, oracle):
    """GPU build, host build and a saved / re-loaded tree agree for a wide
    cloud; gradients flow as for 3-D trees; a batch of the wide tree answers
    like the tree itself."""
    rng = np.random.default_rng(66)
    ref = rng.standard_normal((20000, 6)).astype(np.float32)
    q = rng.standard_normal((3000, 6)).astype(np.float32)
    rt, qt = torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda)
    th = tk().build_kd_tree(rt, build="host", levels=11)
    td = tk().build_kd_tree(rt, build="device", levels=11)
    assert torch.equal(th.shuffled_ind, td.shuffled_ind)
    assert torch.equal(th.structured_points, td.structured_points)
    td.save(tmp_path / "wide.npz")
    tl = tk().load_kd_tree(tmp_path / "wide.npz")
    bd, bi = oracle.brute(ref, q, 9)
    for t in (th, td, tl):
        d, i = t.query(qt, nr_nns_searches=9)
        np.testing.assert_array_equal(d.cpu().numpy(), bd)
        np.testing.assert_array_equal(i.cpu().numpy(), bi)
    qg = qt.clone().requires_grad_(True)
    d, i = td.query(qg, nr_nns_searches=3)
    d.sum().backward()
    assert torch.allclose(qg.grad, 2 * (qg[:, None] - rt[i.long()]).sum(1))
    from torch_kdtree_gb300.batched import BatchedKDTrees
    b = BatchedKDTrees([rt], [4], [10])
    (db,), (ib,) = b.query([qt[:10]])
    d4, i4 = td.query(qt[:10], nr_nns_searches=4)
    assert torch.equal(db, d4) and torch.equal(ib, i4)


def _non_finite_rows(q):
    """Rows whose distances are +inf to every point (infinite coordinates, or
    squares that overflow): every candidate ties at +inf, so the answer is the
    k lowest original indices."""
    q[3, 0] = np.inf
    q[4, 0] = -np.inf
    q[5, :] = 1e20
    q[6, 0], q[6, 1] = np.inf, -np.inf
    q[7, 0] = 3e19
    return q


@pytest.mark.parametrize("dims", [3, 5])
def test_infinite_and_overflowing_queries(dims, oracle):
    rng = np.random.default_rng(70 + dims)
    ref = rng.standard_normal((5000, dims)).astype(np.float32)
    q = _non_finite_rows(rng.standard_normal((400, dims)).astype(np.float32))
    bd, bi = oracle.brute(ref, q, 6)
    assert np.isinf(bd[3:8]).all() and (bi[3:8] == np.arange(6)).all()
    shapes = [dict(), dict(threads_per_query=1), dict(threads_per_query=32), dict(threads_per_query=1, prune_boxes=0)]
    if dims == 3:
        shapes.append(dict(traversal=2))
    for opts in shapes:
        d, i = gpu_query(ref, q, 6, levels=8, **opts)
        np.testing.assert_array_equal(d, bd, err_msg=str(opts))
        np.testing.assert_array_equal(i, bi, err_msg=str(opts))


@pytest.mark.parametrize("dims", [3, 6])
def test_infinite_and_huge_reference_points(dims, oracle):
    rng = np.random.default_rng(80 + dims)
    ref = rng.standard_normal((4000, dims)).astype(np.float32)
    ref[5, 0] = np.inf
    ref[9, 1] = -np.inf
    ref[11, :] = 3e19
    q = rng.standard_normal((300, dims)).astype(np.float32)
    q[0, :] = 3e19
    bd, bi = oracle.brute(ref, q, 5)
    assert bi[0, 0] == 11 and bd[0, 0] == 0
    for opts in (dict(), dict(threads_per_query=1), dict(threads_per_query=32, prune_boxes=0)):
        d, i = gpu_query(ref, q, 5, levels=7, **opts)
        np.testing.assert_array_equal(d, bd, err_msg=str(opts))
        np.testing.assert_array_equal(i, bi, err_msg=str(opts))


@pytest.mark.parametrize("n", [1, 2, 3])
def test_trees_of_one_to_three_points(n, oracle):
    rng = np.random.default_rng(90 + n)
    ref = rng.standard_normal((n, 3)).astype(np.float32)
    q = rng.standard_normal((50, 3)).astype(np.float32)
    for k in range(1, n + 1):
        bd, bi = oracle.brute(ref, q, k)
        for opts in (dict(), dict(threads_per_query=32), dict(traversal=2)):
            d, i = gpu_query(ref, q, k, **opts)
            np.testing.assert_array_equal(d, bd, err_msg=str(opts))
            np.testing.assert_array_equal(i, bi, err_msg=str(opts))


def test_concurrent_queries_on_one_tree():
    """Four threads, each on its own stream, query one tree at the same time
    (the tree is read-only; each call has its own workspace)."""
    import threading
    rng = np.random.default_rng(95)
    tree = tk().build_kd_tree(torch.from_numpy(rng.random((200000, 3), dtype=np.float32)).to(cuda))
    qs = [torch.from_numpy(rng.random((150000 + 11 * t, 3), dtype=np.float32)).to(cuda) for t in range(4)]
    ks = [1, 8, 16, 40]
    want = [tree.query(q, nr_nns_searches=k) for q, k in zip(qs, ks)]
    torch.cuda.synchronize()
    got, errors = [None] * 4, []

    def work(t):
        try:
            torch.cuda.set_device(0)
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                for _ in range(3):
                    got[t] = tree.query(qs[t], nr_nns_searches=ks[t])
            s.synchronize()
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for (wd, wi), (d, i) in zip(want, got):
        assert torch.equal(d, wd) and torch.equal(i, wi)


def test_random_configurations(oracle):
    """A seeded sweep over combinations the targeted tests take one at a time:
    dims 1-8, float32 / float64, cloud and batch sizes from 1 up, any k <= n,
    any depth, lanes per query, forced binning (cost-class order on small
    batches), box pruning, traversal and shared-memory staging; every answer
    bit-exact against the exhaustive search."""
    rng = np.random.default_rng(20260)
    for case in range(120):
        dims = int(rng.integers(1, 9))
        dtype = np.float32 if rng.random() < 0.7 else np.float64
        n = int(rng.choice([2, 17, 300, 2500, 5000]))
        nq = int(rng.choice([1, 3, 64, 700, 2000]))
        k = int(rng.integers(1, min(n, 128) + 1))
        levels = int(rng.integers(1, int(np.log2(n)) + 1))  # the build wants 2^levels <= n
        tpq = int(rng.choice([0, 1, 4, 8, 32]))
        opts = dict(threads_per_query=tpq, bin_queries=int(rng.choice([-1, 0, 1])),
                    prune_boxes=int(rng.integers(0, 2)), traversal=int(rng.choice([0, 1, 2])),
                    smem_levels=int(rng.choice([-1, 0, 4])))
        scale = float(rng.choice([1e-3, 1.0, 1e3]))
        ref = (rng.standard_normal((n, dims)) * scale).astype(dtype)
        q = (rng.standard_normal((nq, dims)) * scale * 1.3).astype(dtype)
        if n > 20:
            ref[rng.integers(0, n, n // 10)] = ref[rng.integers(0, n, n // 10)]  # duplicates: ties
        bd, bi = oracle.brute(ref, q, k)
        d, i = gpu_query(ref, q, k, levels=levels, **opts)
        msg = f"case {case}: dims={dims} {np.dtype(dtype).name} n={n} nq={nq} k={k} L={levels} {opts}"
        np.testing.assert_array_equal(d, bd, err_msg=msg)
        np.testing.assert_array_equal(i, bi, err_msg=msg)
