"""GPU parity of the exhaustive search (nn_distance, tk_nn_distance):
bit-exact against the oracle's exhaustive search, and identical to the
KD-tree query on the same inputs."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def tk():
    import torch_kdtree_gb300
    return torch_kdtree_gb300


@pytest.mark.parametrize("d", [1, 2, 3, 4, 5, 8, 17, 32, 64, 128])
@pytest.mark.parametrize("k", [1, 3, 16, 32, 100])
def test_exact_mode_matches_oracle(d, k, oracle):
    rng = np.random.default_rng(d * 1000 + k)
    n = 6000 if d <= 32 else 3000
    ref = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((700, d)).astype(np.float32)
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k)
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


@pytest.mark.parametrize("d", [1, 2, 3, 5, 8, 17, 40, 128])
def test_float64(d, oracle):
    """FP64 stays FP64 end to end, at any dimension."""
    rng = np.random.default_rng(40 + d)
    ref = rng.standard_normal((5000, d))
    q = rng.standard_normal((500, d))
    for k in (1, 7, 40):
        dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k)
        assert dd.dtype == torch.float64
        bd, bi = oracle.brute(ref, q, k)
        np.testing.assert_array_equal(dd.cpu().numpy(), bd)
        np.testing.assert_array_equal(ii.cpu().numpy(), bi)
    if d in (5, 40):  # gradients in float64 as well
        r = torch.from_numpy(ref).to(cuda).requires_grad_(True)
        qq = torch.from_numpy(q).to(cuda).requires_grad_(True)
        dd, ii = tk().nn_distance(r, qq, 7)
        w = torch.rand_like(dd)
        (dd * w).sum().backward()
        r2 = r.detach().clone().requires_grad_(True)
        q2 = qq.detach().clone().requires_grad_(True)
        ((q2[:, None] - r2[ii.long()]) ** 2).sum(-1).mul(w).sum().backward()
        assert torch.allclose(qq.grad, q2.grad, rtol=1e-12, atol=1e-12)
        assert torch.allclose(r.grad, r2.grad, rtol=1e-12, atol=1e-12)


def test_brute_equals_kdtree():
    g = torch.Generator().manual_seed(3)
    ref = torch.rand(65536, 3, generator=g).to(cuda)
    q = torch.rand(8192, 3, generator=g).to(cuda)
    for k in (1, 16):
        bd, bi = tk().nn_distance(ref, q, k)
        kd, ki = tk().build_kd_tree(ref).query(q, nr_nns_searches=k)
        assert torch.equal(bd, kd) and torch.equal(bi, ki)


def test_duplicates_and_many_slices(oracle):
    """5% exact duplicates; few queries so the reference set is sliced across
    many blocks and the per-slice lists are merged."""
    rng = np.random.default_rng(77)
    ref = rng.standard_normal((200_000, 8)).astype(np.float32)
    m = 10_000
    perm = rng.permutation(len(ref))
    ref[perm[:m]] = ref[perm[m:2 * m]]
    q = ref[rng.integers(0, len(ref), 64)] + np.float32(0)
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), 32)
    bd, bi = oracle.brute(ref, q, 32)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


def test_brute_backward_matches_torch():
    g = torch.Generator().manual_seed(5)
    for d in (3, 8, 32):
        ref = torch.randn(4000, d, generator=g).to(cuda).requires_grad_(True)
        q = torch.randn(3000, d, generator=g).to(cuda).requires_grad_(True)
        w = torch.rand(3000, 4, generator=g).to(cuda)
        dists, inds = tk().nn_distance(ref, q, 4)
        (0.5 * (dists * w).sum()).backward()
        q2 = q.detach().clone().requires_grad_(True)
        r2 = ref.detach().clone().requires_grad_(True)
        d2 = torch.sum((q2[:, None] - r2[inds.long()]) ** 2, -1)
        (0.5 * (d2 * w).sum()).backward()
        assert torch.allclose(q.grad, q2.grad, rtol=1e-4, atol=1e-4)
        assert torch.allclose(ref.grad, r2.grad, rtol=1e-4, atol=1e-4)


def test_errors():
    ref = torch.randn(10, 3, device=cuda)
    with pytest.raises(Exception):
        tk().nn_distance(ref, torch.randn(4, 3, device=cuda), 11)
    with pytest.raises(Exception):
        tk().nn_distance(ref, torch.randn(4, 2, device=cuda), 1)
    with pytest.raises(Exception):
        tk().nn_distance(ref, torch.randn(4, 3, device=cuda, dtype=torch.float64), 1)


@pytest.mark.parametrize("mode", ["tf32", "bf16_split"])
@pytest.mark.parametrize("d", [3, 8, 17, 32, 64])
@pytest.mark.parametrize("k", [1, 16, 32])
def test_tensor_core_modes_are_exact(mode, d, k, oracle):
    """Tensor-core candidate search + exact re-rank (+ exact fallback for
    uncertified queries) returns the exact answer, bit for bit."""
    rng = np.random.default_rng(1000 + 10 * d + k)
    ref = rng.standard_normal((20000, d)).astype(np.float32)
    m = 1000
    perm = rng.permutation(len(ref))
    ref[perm[:m]] = ref[perm[m:2 * m]]  # 5% exact duplicates
    q = rng.standard_normal((3000, d)).astype(np.float32)
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k, mode=mode)
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


@pytest.mark.parametrize("mode", ["tf32", "bf16_split"])
@pytest.mark.parametrize("d", [3, 17, 40])
@pytest.mark.parametrize("k", [33, 64])
def test_tensor_core_large_k(mode, d, k, oracle):
    """k above 32: the mma.sync candidate search with a 128-key over-fetch and
    the two-register re-rank; d = 40 also leaves the tcgen05 path's depth."""
    rng = np.random.default_rng(8800 + d + k)
    ref = rng.standard_normal((30000, d)).astype(np.float32)
    ref[rng.permutation(30000)[:500]] = ref[:500]  # exact duplicates
    q = rng.standard_normal((700, d)).astype(np.float32)
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k, mode=mode)
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)
    if d == 40:  # too big for the candidate search's shared memory: every query exact
        from torch_kdtree_gb300 import _lib
        from torch_kdtree_gb300._lib import LIB
        from torch_kdtree_gb300.nn_distance import _BRUTE_MODES, _stream_ptr
        m = _BRUTE_MODES[mode]
        r_t, q_t = torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda)
        wsb = LIB.tk_nn_distance_workspace_size(len(ref), len(q), d, k, _lib.TK_F32, m)
        ws = torch.empty(wsb, dtype=torch.uint8, device=cuda)
        d2 = torch.empty(len(q), k, device=cuda)
        i2 = torch.empty(len(q), k, dtype=torch.int32, device=cuda)
        _lib.check(LIB.tk_nn_distance(r_t.data_ptr(), len(ref), q_t.data_ptr(), len(q), d, k, _lib.TK_F32, m,
                                      d2.data_ptr(), i2.data_ptr(), ws.data_ptr(), wsb, _stream_ptr(cuda)))
        torch.cuda.synchronize()
        import ctypes
        flags, rec = ctypes.c_int(-1), ctypes.c_int(-1)
        _lib.check(LIB.tk_nn_distance_report(ws.data_ptr(), len(ref), len(q), d, k, _lib.TK_F32, m,
                                             ctypes.byref(flags), ctypes.byref(rec)))
        assert flags.value == 0 and rec.value == len(q)
        np.testing.assert_array_equal(d2.cpu().numpy(), bd)
        np.testing.assert_array_equal(i2.cpu().numpy(), bi)


@pytest.mark.parametrize("mode", ["tf32", "bf16_split"])
@pytest.mark.parametrize("k", [8, 16, 32])
@pytest.mark.parametrize("data", ["normal", "repeated", "grid"])
def test_tensor_core_sampled_threshold_slices(mode, k, data, oracle):
    """Slices long enough (70,000 refs, 8 slices of ~34 tiles) that the
    candidate kernel first samples a threshold: on N(0,1) data, on 300
    distinct points repeated (every tile overflows the hit buffers and is
    redone in 32-column steps) and on an integer grid (exact distance ties).
    The answer must stay the exhaustive search's, bit for bit."""
    rng = np.random.default_rng(4100 + k)
    d = 16
    if data == "normal":
        ref = rng.standard_normal((70000, d)).astype(np.float32)
    elif data == "repeated":
        ref = rng.standard_normal((300, d)).astype(np.float32)[rng.integers(0, 300, 70000)]
    else:
        ref = rng.integers(-3, 4, (70000, d)).astype(np.float32)
    q = rng.standard_normal((600, d)).astype(np.float32)
    if data == "grid":
        q = np.rint(q)  # integer distances: many exact ties
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k, mode=mode)
    bd, bi = oracle.brute(ref, q, k)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


@pytest.mark.parametrize("mode", ["tf32", "bf16_split"])
@pytest.mark.parametrize("n", [1, 7, 255, 256, 257, 513])
@pytest.mark.parametrize("nq", [1, 5, 129])
def test_tensor_core_edge_sizes(mode, n, nq, oracle):
    """Single, partial and exactly-full 256-reference tiles, query blocks of
    1, 5 and 129 rows (one row past a 128-row block), k up to 32 and at most
    n: slices far too short for the sampled threshold, the last tile's
    column bound, padding rows of both operands."""
    rng = np.random.default_rng(7000 + n + nq)
    d = 12
    ref = rng.standard_normal((n, d)).astype(np.float32)
    q = rng.standard_normal((nq, d)).astype(np.float32)
    for k in sorted({1, min(n, 5), min(n, 32)}):
        dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k, mode=mode)
        bd, bi = oracle.brute(ref, q, k)
        np.testing.assert_array_equal(dd.cpu().numpy(), bd)
        np.testing.assert_array_equal(ii.cpu().numpy(), bi)


@pytest.mark.parametrize("mode", ["tf32", "bf16_split"])
def test_tensor_core_fallback_on_massive_ties(mode, oracle):
    """64 distinct points repeated ~300 times: candidate lists cannot separate
    the k-th neighbour from the rest, the certificate fails and the exact
    fallback must produce the answer."""
    rng = np.random.default_rng(7)
    base = rng.standard_normal((64, 16)).astype(np.float32)
    ref = base[rng.integers(0, 64, 20000)]
    q = rng.standard_normal((500, 16)).astype(np.float32)
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), 20, mode=mode)
    bd, bi = oracle.brute(ref, q, 20)
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


def test_auto_mode_picks_a_mode_and_stays_exact(tmp_path, monkeypatch, oracle):
    """mode="auto" times the modes once (cached) and returns the exact answer."""
    import torch_kdtree_gb300.autotune as at
    from torch_kdtree_gb300 import nn_distance
    monkeypatch.setattr(at, "CACHE_PATH", str(tmp_path / "cache.json"))
    rng = np.random.default_rng(44)
    for d, dtype in ((32, np.float32), (3, np.float32), (3, np.float64)):
        ref = rng.standard_normal((20000, d)).astype(dtype)
        q = rng.standard_normal((700, d)).astype(dtype)
        rt, qt = torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda)
        mode = at.autotune_brute(rt, qt, 8)
        assert mode in (("exact",) if dtype == np.float64 else ("exact", "tf32", "bf16_split"))
        dd, ii = nn_distance(rt, qt, 8, mode="auto")
        bd, bi = oracle.brute(ref, q, 8)
        np.testing.assert_array_equal(dd.cpu().numpy(), bd)
        np.testing.assert_array_equal(ii.cpu().numpy(), bi)
    import json
    assert len(json.load(open(tmp_path / "cache.json"))) == 3


@pytest.mark.parametrize("mode", ["exact", "tf32", "bf16_split"])
def test_infinite_and_overflowing_queries(mode, oracle):
    """Rows whose distances are +inf to every reference (infinite coordinates,
    or squares that overflow) tie at +inf: the k lowest indices, in every mode
    (the tensor-core modes cannot certify them and fall back to exact)."""
    rng = np.random.default_rng(77)
    ref = rng.standard_normal((20000, 8)).astype(np.float32)
    q = rng.standard_normal((600, 8)).astype(np.float32)
    q[3, 0] = np.inf
    q[4, 0] = -np.inf
    q[5, :] = 1e20
    q[6, 0], q[6, 1] = np.inf, -np.inf
    q[7, 0] = 3e19
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), 5, mode=mode)
    bd, bi = oracle.brute(ref, q, 5)
    assert np.isinf(bd[3:8]).all() and (bi[3:8] == np.arange(5)).all()
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


@pytest.mark.parametrize("mode", ["exact", "tf32", "bf16_split"])
def test_infinite_and_huge_references(mode, oracle):
    """References with infinite coordinates or norms beyond the tensor-core
    range: the tensor-core modes certify nothing and fall back to exact; the
    answers equal the oracle's (such references sit at distance +inf)."""
    rng = np.random.default_rng(78)
    ref = rng.standard_normal((20000, 8)).astype(np.float32)
    ref[5, 2] = np.inf
    ref[9, 0] = -np.inf
    ref[11, :] = 3e19
    q = rng.standard_normal((700, 8)).astype(np.float32)
    q[0, :] = 3e19  # next to ref 11: distance 0 there, +inf to everything else
    dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), 4, mode=mode)
    bd, bi = oracle.brute(ref, q, 4)
    assert bi[0, 0] == 11 and bd[0, 0] == 0
    np.testing.assert_array_equal(dd.cpu().numpy(), bd)
    np.testing.assert_array_equal(ii.cpu().numpy(), bi)


def test_random_configurations(oracle):
    """A seeded sweep over exhaustive-search shapes: dims 1-64, k up to 64 and
    n, query counts from 1 up, every mode (tensor-core modes for float32),
    duplicates; every answer bit-exact against the oracle."""
    rng = np.random.default_rng(31337)
    for case in range(60):
        d = int(rng.choice([1, 2, 3, 5, 8, 12, 16, 24, 31, 32, 33, 39, 40, 47, 48, 64]))
        n = int(rng.choice([1, 5, 64, 257, 1500, 4000]))
        nq = int(rng.choice([1, 7, 129, 500]))
        k = int(rng.integers(1, min(n, 64) + 1))
        mode = str(rng.choice(["exact", "tf32", "bf16_split"]))
        dtype = np.float64 if (mode == "exact" and rng.random() < 0.3) else np.float32
        ref = (rng.standard_normal((n, d)) * float(rng.choice([1e-2, 1.0, 1e2]))).astype(dtype)
        if n > 10:
            ref[rng.integers(0, n, n // 8)] = ref[rng.integers(0, n, n // 8)]
        q = rng.standard_normal((nq, d)).astype(dtype)
        dd, ii = tk().nn_distance(torch.from_numpy(ref).to(cuda), torch.from_numpy(q).to(cuda), k, mode=mode)
        bd, bi = oracle.brute(ref, q, k)
        msg = f"case {case}: d={d} n={n} nq={nq} k={k} {mode} {np.dtype(dtype).name}"
        np.testing.assert_array_equal(dd.cpu().numpy(), bd, err_msg=msg)
        np.testing.assert_array_equal(ii.cpu().numpy(), bi, err_msg=msg)
