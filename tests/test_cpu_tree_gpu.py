"""CPU and GPU queries of the same host-built tree give the same bits, and a
tree built on the GPU (no host layout) refuses CPU queries."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_cpu_and_gpu_queries_of_one_tree_are_identical():
    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300._lib import LIB, check
    from torch_kdtree_gb300.synthetic import cube_and_sphere
    ref, q = cube_and_sphere(n_ref=1 << 20, n_query=1 << 15, seed=11)
    k = 16
    tree = tk.build_kd_tree(torch.from_numpy(ref).cuda(), levels=16, build="host")
    gd, gi = tree.query(torch.from_numpy(q).cuda(), nr_nns_searches=k)
    cd = np.empty((len(q), k), np.float32)
    ci = np.empty((len(q), k), np.int32)
    check(LIB.tk_tree_query_cpu(tree._tree.handle, q.ctypes.data, len(q), k, cd.ctypes.data, ci.ctypes.data, 0))
    np.testing.assert_array_equal(gd.cpu().numpy(), cd)
    np.testing.assert_array_equal(gi.cpu().numpy(), ci)
    ctree = tk.build_kd_tree(torch.from_numpy(ref), device="cpu", levels=16)
    d2, i2 = ctree.query(torch.from_numpy(q), nr_nns_searches=k)
    np.testing.assert_array_equal(d2.numpy(), cd)
    np.testing.assert_array_equal(i2.numpy(), ci)


def test_gpu_built_tree_refuses_cpu_query():
    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL
    ref = torch.randn(1000, 3, device="cuda")
    tree = tk.build_kd_tree(ref, build="device")
    q = np.zeros((4, 3), np.float32)
    d = np.empty((4, 2), np.float32)
    i = np.empty((4, 2), np.int32)
    assert LIB.tk_tree_query_cpu(tree._tree.handle, q.ctypes.data, 4, 2, d.ctypes.data, i.ctypes.data, 0) == TK_EINVAL
    assert b"host layout" in LIB.tk_last_error()
