"""Tree files (TorchKDTree.save / load_kd_tree) and the two-way brute-force
search (nn_distance_bidirectional) on the GPU."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("build", ["host", "device"])
def test_save_load_round_trip(tmp_path, dtype, build, oracle):
    import torch_kdtree_gb300 as tk
    rng = np.random.default_rng(40)
    ref_np = rng.standard_normal((20000, 3))
    q_np = rng.standard_normal((1500, 3))
    ref = torch.from_numpy(ref_np).to(cuda, dtype)
    q = torch.from_numpy(q_np).to(cuda, dtype)
    tree = tk.build_kd_tree(ref, levels=10, build=build)
    path = tmp_path / "tree.npz"
    tree.save(path)
    loaded = tk.load_kd_tree(path)
    assert loaded.built_on == "file" and loaded.levels == 10 and loaded.dtype == dtype
    assert torch.equal(loaded.shuffled_ind, tree.shuffled_ind)
    assert torch.equal(loaded.structured_points, tree.structured_points)
    assert torch.equal(loaded.points_ref_bak, ref)  # the original order is restored
    for k in (1, 7, 32):
        d0, i0 = tree.query(q, nr_nns_searches=k)
        d1, i1 = loaded.query(q, nr_nns_searches=k)
        assert torch.equal(d0, d1) and torch.equal(i0, i1)
    bd, bi = oracle.brute(ref.cpu().numpy(), q.cpu().numpy(), 7)
    d1, i1 = loaded.query(q, nr_nns_searches=7)
    np.testing.assert_array_equal(d1.cpu().numpy(), bd)
    np.testing.assert_array_equal(i1.cpu().numpy(), bi)


def test_loaded_tree_gradients_and_errors(tmp_path):
    import torch_kdtree_gb300 as tk
    ref = torch.randn(500, 3, device=cuda)
    tree = tk.build_kd_tree(ref)
    tree.save(tmp_path / "t.npz")
    loaded = tk.load_kd_tree(tmp_path / "t.npz")
    q = torch.randn(40, 3, device=cuda, requires_grad=True)
    d, i = loaded.query(q, nr_nns_searches=3)
    d.sum().backward()
    expect = 2 * (q[:, None] - ref[i.long()]).sum(1)
    assert torch.allclose(q.grad, expect)
    z = dict(np.load(tmp_path / "t.npz"))
    z["shuffled_ind"] = z["shuffled_ind"].copy()
    z["shuffled_ind"][0] = z["shuffled_ind"][1]
    np.savez(tmp_path / "bad.npz", **z)
    with pytest.raises(Exception):
        tk.load_kd_tree(tmp_path / "bad.npz")
    z = dict(np.load(tmp_path / "t.npz"))
    z["format"] = np.array("something else")
    np.savez(tmp_path / "other.npz", **z)
    with pytest.raises(ValueError):
        tk.load_kd_tree(tmp_path / "other.npz")


@pytest.mark.parametrize("mode", ["exact", "tf32"])
def test_bidirectional_nn_distance(mode, oracle):
    import torch_kdtree_gb300 as tk
    rng = np.random.default_rng(41)
    a = rng.standard_normal((3000, 3)).astype(np.float32)
    b = rng.standard_normal((2000, 3)).astype(np.float32)
    at, bt = torch.from_numpy(a).to(cuda), torch.from_numpy(b).to(cuda)
    d1, i1, d2, i2 = tk.nn_distance_bidirectional(at, bt, 2, mode=mode)
    e1, j1 = oracle.brute(b, a, 2)  # every point of a among b
    e2, j2 = oracle.brute(a, b, 2)
    np.testing.assert_array_equal(d1.cpu().numpy(), e1)
    np.testing.assert_array_equal(i1.cpu().numpy(), j1)
    np.testing.assert_array_equal(d2.cpu().numpy(), e2)
    np.testing.assert_array_equal(i2.cpu().numpy(), j2)
    # chamfer loss gradients flow to both clouds
    at.requires_grad_(True)
    bt.requires_grad_(True)
    d1, _, d2, _ = tk.nn_distance_bidirectional(at, bt, 1, mode=mode)
    (d1.mean() + d2.mean()).backward()
    assert at.grad is not None and bt.grad is not None
    assert torch.isfinite(at.grad).all() and torch.isfinite(bt.grad).all()
