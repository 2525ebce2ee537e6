"""The hand-written backward (tk_knn_backward) against the reference's
torch-indexed gradient, FP64 central finite differences, and itself
(bitwise determinism)."""
import pytest
import torch

pytestmark = pytest.mark.gpu

cuda = torch.device("cuda")


def tk():
    import torch_kdtree_gb300
    return torch_kdtree_gb300


def torch_indexed_grads(q, ref, inds, w):
    """The reference's gradient path: re-gather and autograd through indexing
    (torch_kdtree/nn_distance.py:111-112)."""
    q = q.detach().clone().requires_grad_(True)
    ref = ref.detach().clone().requires_grad_(True)
    d = torch.sum((q[:, None] - ref[inds.long()]) ** 2, dim=-1)
    (0.5 * (d * w).sum()).backward()
    return q.grad, ref.grad


@pytest.mark.parametrize("dtype,tol", [(torch.float32, 1e-5), (torch.float64, 1e-12)])
@pytest.mark.parametrize("d", [1, 2, 3, 5, 8, 12, 40])
def test_matches_torch_indexed_gradient(dtype, tol, d):
    g = torch.Generator(device="cpu").manual_seed(7)
    ref = torch.randn(20000, d, generator=g, dtype=dtype).to(cuda).requires_grad_(True)
    q = torch.randn(30000, d, generator=g, dtype=dtype).to(cuda).requires_grad_(True)
    k = 8
    w = torch.rand(30000, k, generator=g, dtype=dtype).to(cuda)
    if d <= 8:
        dists, inds = tk().build_kd_tree(ref).query(q, nr_nns_searches=k)
    else:  # KD trees stop at 8 dims; the exhaustive search has the same backward
        dists, inds = tk().nn_distance(ref, q, k)
    (0.5 * (dists * w).sum()).backward()
    gq_t, gr_t = torch_indexed_grads(q, ref, inds, w)
    scale_q = gq_t.abs().max().item()
    scale_r = gr_t.abs().max().item()
    assert (q.grad - gq_t).abs().max().item() <= tol * scale_q * 10
    assert (ref.grad - gr_t).abs().max().item() <= tol * scale_r * 10


def test_backward_is_bitwise_deterministic():
    g = torch.Generator(device="cpu").manual_seed(8)
    ref = torch.randn(100000, 3, generator=g).to(cuda)
    q = torch.randn(100000, 3, generator=g).to(cuda)
    w = torch.rand(100000, 8, generator=g).to(cuda)
    outs = []
    for _ in range(3):
        r = ref.clone().requires_grad_(True)
        qq = q.clone().requires_grad_(True)
        dists, _ = tk().build_kd_tree(r).query(qq, nr_nns_searches=8)
        (0.5 * (dists * w).sum()).backward()
        outs.append((qq.grad.clone(), r.grad.clone()))
    for gq, gr in outs[1:]:
        assert torch.equal(gq, outs[0][0])
        assert torch.equal(gr, outs[0][1])


def test_finite_differences_fp64():
    """Central differences (step 1e-4, FP64) of loss = 0.5 * sum(dists * w)
    with the neighbour lists held fixed, on a 4,096-point subset."""
    g = torch.Generator(device="cpu").manual_seed(9)
    n = 200_000
    ref = torch.randn(n, 3, generator=g).to(cuda).requires_grad_(True)
    q = torch.randn(n, 3, generator=g).to(cuda).requires_grad_(True)
    w = torch.rand(n, 8, generator=g).to(cuda)
    dists, inds = tk().build_kd_tree(ref).query(q, nr_nns_searches=8)
    (0.5 * (dists * w).sum()).backward()

    q64 = q.detach().double()
    r64 = ref.detach().double()
    w64 = w.double()
    il = inds.long()

    def loss(qv, rv):
        return 0.5 * (torch.sum((qv[:, None] - rv[il]) ** 2, -1) * w64).sum()

    h = 1e-4
    sub = torch.randperm(n, generator=g)[:4096].to(cuda)
    # query coordinates: perturb one coordinate of all subset points at once
    # (their loss terms are independent), per axis
    for c in range(3):
        e = torch.zeros_like(q64)
        e[sub, c] = h
        # per-point contributions: only rows in sub change
        lp = 0.5 * (torch.sum(((q64 + e)[sub][:, None] - r64[il[sub]]) ** 2, -1) * w64[sub]).sum(1)
        lm = 0.5 * (torch.sum(((q64 - e)[sub][:, None] - r64[il[sub]]) ** 2, -1) * w64[sub]).sum(1)
        fd = (lp - lm) / (2 * h)
        an = q.grad[sub, c].double()
        rel = ((an - fd).abs() / fd.abs().clamp_min(1e-2)).max().item()
        assert rel < 1e-3, rel
    # reference coordinates: one point at a time for a smaller subset
    for m in sub[:64].tolist():
        for c in range(3):
            e = torch.zeros_like(r64)
            e[m, c] = h
            fd = ((loss(q64, r64 + e) - loss(q64, r64 - e)) / (2 * h)).item()
            an = ref.grad[m, c].item()
            assert abs(an - fd) <= 1e-3 * max(abs(fd), 1e-3), (m, c, an, fd)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("d", [3, 6, 16])
def test_hub_segments_are_deterministic_and_accurate(d, dtype):
    """Every query shares the same few neighbours (segments of 100,000+ pairs):
    the order-independent fixed-point sums (64-bit integers for float32
    terms, 128-bit for float64; 8 coordinates per pass) give the same bits on
    every run and match a sum in higher precision."""
    g = torch.Generator(device="cpu").manual_seed(9)
    ref = torch.randn(5000, d, generator=g, dtype=dtype)
    ref[:8] = 40.0 + torch.randn(8, d, generator=g, dtype=dtype) * 1e-3  # a far-away cluster of 8 points
    q = 40.0 + torch.randn(120000, d, generator=g, dtype=dtype) * 1e-2    # all queries next to it
    ref, q = ref.to(cuda), q.to(cuda)
    w = torch.rand(120000, 8, generator=g, dtype=dtype).to(cuda)
    outs = []
    for _ in range(3):
        r = ref.clone().requires_grad_(True)
        qq = q.clone().requires_grad_(True)
        dists, inds = tk().nn_distance(r, qq, 8)
        (0.5 * (dists * w).sum()).backward()
        outs.append(r.grad.clone())
    assert (inds.long() < 8).all()
    for gr in outs[1:]:
        assert torch.equal(gr, outs[0])
    # the same terms summed in higher precision (FP64 for float32 terms; for
    # float64 terms, FP64 of the rounded terms on the CPU in a fixed order)
    il = inds.long().cpu()
    terms = (w.double().cpu()[..., None] * (ref.double().cpu()[il] - q.double().cpu()[:, None]))
    exact = torch.zeros(ref.shape, dtype=torch.float64).index_add_(0, il.reshape(-1), terms.reshape(-1, d))
    err = (outs[0].double().cpu() - exact).abs().max().item()
    # fixed-point sums: one rounding of a sum far more precise than the terms
    assert err <= (1e-5 if dtype == torch.float32 else 1e-12) * exact.abs().max().item()


def test_no_queries_gives_zero_reference_gradient():
    from torch_kdtree_gb300.autograd import knn_backward
    ref = torch.randn(100, 3, device=cuda)
    q = torch.empty(0, 3, device=cuda)
    idx = torch.empty(0, 4, dtype=torch.int32, device=cuda)
    g = torch.empty(0, 4, device=cuda)
    gq, gr = knn_backward(q, ref, idx, g, True, True)
    assert gq.shape == (0, 3) and torch.equal(gr, torch.zeros_like(ref))
