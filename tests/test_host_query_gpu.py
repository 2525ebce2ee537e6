"""GPU parity of the host-buffer query (tk_tree_query_host): queries and
results in host memory, the results written by the query kernel directly
(pinned buffers) or downloaded from device staging.  Bar: bit-identical to
the device-resident query (itself bit-exact against the oracle)."""
import threading

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def tk():
    import torch_kdtree_gb300
    return torch_kdtree_gb300


def host_buffers(nq, k, dtype, pinned):
    d = torch.empty(nq, k, dtype=dtype)
    i = torch.empty(nq, k, dtype=torch.int32)
    return (d.pin_memory(), i.pin_memory()) if pinned else (d, i)


@pytest.mark.parametrize("dims,dtype", [(3, torch.float32), (2, torch.float64), (6, torch.float32),
                                        (8, torch.float64), (1, torch.float32)])
@pytest.mark.parametrize("pinned", [True, False])
def test_host_query_equals_device_query(dims, dtype, pinned, oracle):
    rng = np.random.default_rng(dims)
    ref = rng.standard_normal((30000, dims))
    q = rng.standard_normal((70001, dims)) * 1.1
    tree = tk().build_kd_tree(torch.from_numpy(ref).to(dtype).to(cuda))
    q_host = torch.from_numpy(q).to(dtype)
    if pinned:
        q_host = q_host.pin_memory()
    for k in (1, 16, 128):
        dd, di = tree.query(q_host.to(cuda), nr_nns_searches=k)
        hd, hi = host_buffers(len(q), k, dtype, pinned)
        d, i = tree.query(q_host, nr_nns_searches=k, result_dists=hd, result_idx=hi)
        assert d.device.type == "cpu" and i.device.type == "cpu"
        assert d.data_ptr() == hd.data_ptr() and i.data_ptr() == hi.data_ptr()
        assert torch.equal(d, dd.cpu()) and torch.equal(i, di.cpu())
    bd, bi = oracle.brute(ref.astype(q_host.numpy().dtype), q_host[:2000].numpy(), 16)
    d, i = tree.query(q_host[:2000], nr_nns_searches=16, result_dists=torch.empty(2000, 16, dtype=dtype),
                      result_idx=torch.empty(2000, 16, dtype=torch.int32))
    np.testing.assert_array_equal(d.numpy(), bd)
    np.testing.assert_array_equal(i.numpy(), bi)


@pytest.mark.parametrize("transfer", [0, 1, 2])
@pytest.mark.parametrize("k", [5, 16, 32])
def test_host_query_transfers(transfer, k):
    """Direct (kernel writes pinned host memory), staged and auto give the
    device query's results; direct refuses pageable result buffers."""
    from torch_kdtree_gb300 import _lib
    from torch_kdtree_gb300.nn_distance import knn_query_host
    rng = np.random.default_rng(7)
    ref = torch.from_numpy(rng.random((50000, 3), dtype=np.float32)).to(cuda)
    nq = 200003
    q = torch.from_numpy(rng.random((nq, 3), dtype=np.float32))
    tree = tk().build_kd_tree(ref)
    dd, di = tree.query(q.to(cuda), nr_nns_searches=k)
    hd, hi = host_buffers(nq, k, torch.float32, True)
    knn_query_host(tree._tree, q.pin_memory(), k, hd, hi, cuda, tree.query_opts, transfer)
    assert torch.equal(hd, dd.cpu()) and torch.equal(hi, di.cpu())
    # odd row offsets (views into a larger pinned buffer): unaligned rows take the scalar stores
    big_d = torch.empty(nq * k + 1).pin_memory()
    big_i = torch.empty(nq * k + 1, dtype=torch.int32).pin_memory()
    vd, vi = big_d[1:].view(nq, k), big_i[1:].view(nq, k)
    knn_query_host(tree._tree, q.pin_memory(), k, vd, vi, cuda, tree.query_opts, transfer)
    assert torch.equal(vd, dd.cpu()) and torch.equal(vi, di.cpu())
    if transfer == _lib.TK_HOST_DIRECT:
        pd, pi = host_buffers(nq, k, torch.float32, False)
        with pytest.raises(RuntimeError):
            knn_query_host(tree._tree, q, k, pd, pi, cuda, tree.query_opts, transfer)


def test_host_query_edge_cases():
    from torch_kdtree_gb300 import _lib
    rng = np.random.default_rng(8)
    ref = torch.from_numpy(rng.random((1000, 3), dtype=np.float32)).to(cuda)
    tree = tk().build_kd_tree(ref)
    # no queries
    d, i = tree.query(torch.empty(0, 3), nr_nns_searches=4, result_dists=torch.empty(0, 4),
                      result_idx=torch.empty(0, 4, dtype=torch.int32))
    assert d.shape == (0, 4) and i.shape == (0, 4)
    # k = n, one query
    q = torch.rand(1, 3)
    small = tk().build_kd_tree(ref[:100])
    d, i = small.query(q, nr_nns_searches=100, result_dists=torch.empty(1, 100),
                       result_idx=torch.empty(1, 100, dtype=torch.int32))
    assert sorted(i[0].tolist()) == list(range(100))
    # errors as the device query
    with pytest.raises(RuntimeError):
        small.query(q, nr_nns_searches=101, result_dists=torch.empty(1, 101),
                    result_idx=torch.empty(1, 101, dtype=torch.int32))
    with pytest.raises(AssertionError):
        tree.query(q, nr_nns_searches=2, result_dists=torch.empty(1, 3), result_idx=torch.empty(1, 2, dtype=torch.int32))
    with pytest.raises(AssertionError):
        tree.query(q.double(), nr_nns_searches=2, result_dists=torch.empty(1, 2),
                   result_idx=torch.empty(1, 2, dtype=torch.int32))
    # the C entry point refuses bad arguments without touching the GPU
    rc = _lib.LIB.tk_tree_query_host(tree._tree.handle, q.data_ptr(), 1, 2, None, None, None, 0, None)
    assert rc == _lib.TK_EINVAL
    rc = _lib.LIB.tk_tree_query_host(tree._tree.handle, q.data_ptr(), 1, 2, q.data_ptr(), q.data_ptr(), None, 7,
                                     None)
    assert rc == _lib.TK_EINVAL


def test_host_query_accepts_device_buffers_too():
    """The host-buffer entry point copies with the kind inferred from the
    pointers, so device (or mixed) buffers work as well."""
    from torch_kdtree_gb300.nn_distance import knn_query_host
    rng = np.random.default_rng(12)
    ref = torch.from_numpy(rng.random((20000, 3), dtype=np.float32)).to(cuda)
    tree = tk().build_kd_tree(ref)
    q = torch.from_numpy(rng.random((5000, 3), dtype=np.float32))
    dd, di = tree.query(q.to(cuda), nr_nns_searches=6)
    d_dev = torch.empty(5000, 6, device=cuda)
    i_dev = torch.empty(5000, 6, dtype=torch.int32, device=cuda)
    knn_query_host(tree._tree, q.to(cuda), 6, d_dev, i_dev, cuda, tree.query_opts)
    assert torch.equal(d_dev, dd) and torch.equal(i_dev, di)
    d_h, i_h = host_buffers(5000, 6, torch.float32, False)
    knn_query_host(tree._tree, q.to(cuda), 6, d_h, i_h, cuda, tree.query_opts)
    assert torch.equal(d_h, dd.cpu()) and torch.equal(i_h, di.cpu())


def test_host_query_waits_for_earlier_stream_work():
    """Queries copied device -> pinned host asynchronously on the current
    stream just before the call: the pipeline's uploads start after that copy."""
    rng = np.random.default_rng(9)
    ref = torch.from_numpy(rng.random((40000, 3), dtype=np.float32)).to(cuda)
    tree = tk().build_kd_tree(ref)
    q_dev = torch.rand(300000, 3, device=cuda)
    dd, di = tree.query(q_dev, nr_nns_searches=5)
    q_pin = torch.zeros(300000, 3).pin_memory()
    for _ in range(3):
        q_dev.mul_(1.0)  # queue some work ahead of the copy
    q_pin.copy_(q_dev, non_blocking=True)
    hd, hi = host_buffers(300000, 5, torch.float32, True)
    d, i = tree.query(q_pin, nr_nns_searches=5, result_dists=hd, result_idx=hi)
    assert torch.equal(d, dd.cpu()) and torch.equal(i, di.cpu())


def test_host_query_threads_share_a_tree():
    rng = np.random.default_rng(10)
    ref = torch.from_numpy(rng.random((60000, 3), dtype=np.float32)).to(cuda)
    tree = tk().build_kd_tree(ref)
    qs = [torch.from_numpy(rng.random((100000 + 17 * t, 3), dtype=np.float32)).pin_memory() for t in range(4)]
    want = [tree.query(q.to(cuda), nr_nns_searches=7) for q in qs]
    got = [None] * 4
    errors = []

    def work(t):
        try:
            torch.cuda.set_device(0)
            with torch.cuda.stream(torch.cuda.Stream()):
                hd, hi = host_buffers(len(qs[t]), 7, torch.float32, True)
                got[t] = tree.query(qs[t], nr_nns_searches=7, result_dists=hd, result_idx=hi)
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=work, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for (wd, wi), (d, i) in zip(want, got):
        assert torch.equal(d, wd.cpu()) and torch.equal(i, wi.cpu())


def test_host_buffers_with_device_queries_and_gradients():
    rng = np.random.default_rng(11)
    ref = torch.from_numpy(rng.random((5000, 3), dtype=np.float32)).to(cuda)
    tree = tk().build_kd_tree(ref, squared_distances=False)
    q = torch.from_numpy(rng.random((3000, 3), dtype=np.float32))
    dd, di = tree.query(q.to(cuda), nr_nns_searches=4)
    # device queries, host results
    hd, hi = host_buffers(3000, 4, torch.float32, False)
    d, i = tree.query(q.to(cuda), nr_nns_searches=4, result_dists=hd, result_idx=hi)
    assert d.device.type == "cpu" and torch.equal(d, dd.cpu()) and torch.equal(i, di.cpu())
    assert torch.equal(hd.sqrt(), dd.cpu())  # the buffers hold squared distances, as the reference's
    # gradient through host buffers: the returned distances are differentiable
    qg = q.clone().requires_grad_(True)
    hd2, hi2 = host_buffers(3000, 4, torch.float32, False)
    d, i = tree.query(qg, nr_nns_searches=4, result_dists=hd2, result_idx=hi2)
    assert d.device.type == "cpu" and torch.equal(i, di.cpu())
    d.sum().backward()
    assert qg.grad is not None and torch.isfinite(qg.grad).all()
