"""GPU tree construction (tk_tree_create_device): the layout must equal the
host build's bit for bit -- point order, original indices, split values and
leaf offsets -- and through it the reference's own layouts (golden fixtures,
whose host-build equality test_abi pins), on tie-free, tie-heavy, signed-zero
and infinite coordinates, every dimension and dtype, and every depth."""
import ctypes

import numpy as np
import pytest
import torch

from golden_util import inputs_of
from test_abi import host_tree, layout_of

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def device_tree(points: np.ndarray, levels: int):
    from torch_kdtree_gb300._lib import LIB
    t = torch.from_numpy(points).to(cuda)
    h = ctypes.c_void_p()
    dt = 0 if points.dtype == np.float32 else 1
    st = LIB.tk_tree_create_device(t.data_ptr(), points.shape[0], points.shape[1], dt, levels, 0,
                                   torch.cuda.current_stream().cuda_stream, ctypes.byref(h))
    return st, h


def both_layouts(points: np.ndarray, levels: int):
    from torch_kdtree_gb300._lib import LIB, check
    n, d = points.shape
    st, hh = host_tree(points, levels)
    check(st)
    st, hd = device_tree(points, levels)
    try:
        check(st)
        return (layout_of(hh, n, d, levels, points.dtype), layout_of(hd, n, d, levels, points.dtype))
    finally:
        LIB.tk_tree_destroy(hh)
        if hd.value:
            LIB.tk_tree_destroy(hd)


def assert_same_layout(points, levels):
    a, b = both_layouts(points, levels)
    for x, y in zip(a, b):
        assert x.dtype == y.dtype
        np.testing.assert_array_equal(x.view(np.uint8), y.view(np.uint8))  # bitwise


def clouds(dtype, d, n, seed):
    rng = np.random.default_rng(seed)
    yield "normal", rng.standard_normal((n, d)).astype(dtype)
    yield "grid", rng.integers(-3, 4, size=(n, d)).astype(dtype)  # heavy coordinate ties
    p = rng.standard_normal((n, d)).astype(dtype)
    p[rng.permutation(n)[: n // 3]] = p[rng.integers(0, n, size=n // 3)]  # exact duplicate points
    yield "dups", p
    z = rng.standard_normal((n, d)).astype(dtype)
    z[rng.random(n) < 0.3, 0] = dtype(0.0)
    z[rng.random(n) < 0.3, 0] = -dtype(0.0)  # signed zeros tie with each other
    yield "signed_zero", z
    w = (rng.standard_normal((n, d)) * 1e3).astype(dtype)
    w[rng.random(n) < 0.02, -1] = np.inf
    w[rng.random(n) < 0.02, 0] = -np.inf
    yield "inf", w


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 8])
def test_device_build_equals_host_build(dtype, d):
    for n in (1, 2, 3, 17, 1000, 65537):
        lmax = max(1, int(np.floor(np.log2(n))) + 1)  # leaf parents need >= 1 point: n >= 2^(L-1)
        for levels in sorted({max(1, min(lmax, x)) for x in (1, 2, 5, lmax - 3, lmax)}):
            for kind, pts in clouds(dtype, d, n, seed=n * 7 + d):
                try:
                    assert_same_layout(pts, levels)
                except AssertionError as e:
                    raise AssertionError(f"{kind} n={n} d={d} L={levels} {dtype.__name__}") from e


def test_device_build_equals_host_build_large():
    from torch_kdtree_gb300.synthetic import cube_and_sphere
    ref, _ = cube_and_sphere(n_ref=1 << 20, n_query=16, seed=3)
    for levels in (13, 16, 19):
        assert_same_layout(ref, levels)


@pytest.mark.parametrize("name", [
    "grid_f32_d1_n1000_q200_k10", "grid_f32_d2_n10000_q300_k20", "grid_f32_d3_n10000_q300_k20",
    "grid_f64_d1_n10000_q300_k20", "grid_f64_d3_n1000_q200_k10", "grid_f32_d3_n30_q20_k5",
    "grid_f64_d2_n5_q5_k1", "levels_f32_d3_n1000_L9", "levels_f32_d3_n1000_L1"])
def test_device_build_matches_reference_layout(name, golden):
    from torch_kdtree_gb300._lib import LIB, check
    case = golden[name]
    ref, _ = inputs_of(case)
    n, d = ref.shape
    L = int(case["levels"])
    st, h = device_tree(ref, L)
    check(st)
    try:
        pts, perm, med, off = layout_of(h, n, d, L, ref.dtype)
    finally:
        LIB.tk_tree_destroy(h)
    np.testing.assert_array_equal(pts, case["structured"])
    np.testing.assert_array_equal(perm, case["perm"])
    np.testing.assert_array_equal(med, case["medians"])
    np.testing.assert_array_equal(off[:-1], case["leaf_off"])


def test_device_built_tree_queries_like_host_built(oracle):
    import torch_kdtree_gb300 as tk
    rng = np.random.default_rng(21)
    ref = rng.standard_normal((50_000, 3)).astype(np.float32)
    q = rng.standard_normal((4000, 3)).astype(np.float32)
    rt, qt = torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda)
    th = tk.build_kd_tree(rt, build="host", levels=12)
    td = tk.build_kd_tree(rt, build="device", levels=12)
    assert th.built_on == "host" and td.built_on == "device"
    assert tk.build_kd_tree(rt).built_on == "device"  # auto picks the GPU for CUDA input
    assert torch.equal(th.shuffled_ind, td.shuffled_ind)
    assert torch.equal(th.structured_points, td.structured_points)
    for k in (1, 16, 100):
        dh, ih = th.query(qt, nr_nns_searches=k)
        dd, id_ = td.query(qt, nr_nns_searches=k)
        assert torch.equal(dh, dd) and torch.equal(ih, id_)
    bd, bi = oracle.brute(ref, q, 16)
    dd, id_ = td.query(qt, nr_nns_searches=16)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(id_.cpu().numpy(), bi)


def test_device_build_errors():
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL
    import torch_kdtree_gb300 as tk
    pts = np.random.default_rng(0).standard_normal((100, 3)).astype(np.float32)
    st, h = device_tree(pts, 8)  # leaf parents at depth 7 need >= 128 points
    assert st == TK_EINVAL and not h.value
    bad = pts.copy()
    bad[37, 1] = np.nan
    st, h = device_tree(bad, 3)
    assert st == TK_EINVAL and b"NaN" in LIB.tk_last_error()
    host = torch.from_numpy(pts)
    h = ctypes.c_void_p()
    st = LIB.tk_tree_create_device(host.data_ptr(), 100, 3, 0, 3, 0, None, ctypes.byref(h))
    assert st == TK_EINVAL  # host memory is refused
    with pytest.raises(Exception):
        tk.build_kd_tree(torch.from_numpy(bad).to(cuda), levels=3)
    with pytest.raises(Exception):
        tk.build_kd_tree(torch.from_numpy(pts).to(cuda), levels=8)
