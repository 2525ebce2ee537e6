"""tk_tree_query_noalloc: the query entry point for callers that cannot
allocate device memory (their memory belongs to another allocator, they bind
through a plain C FFI with no allocator, or cudaMalloc's device-wide
synchronisation is not acceptable on their path).  Its scratch is a static
device array inside the library, shared by every call.

Checked through the C ABI against tk_tree_query on two calls in a row (the
second call finds the first call's leftovers in the shared scratch), plus the
size limit.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _tree(lib, pts, levels):
    h = ctypes.c_void_p()
    st = lib.tk_tree_create(pts.ctypes.data, pts.shape[0], pts.shape[1], 0, levels,
                            torch.cuda.current_device(), 0, ctypes.byref(h))
    assert st == 0, lib.tk_last_error()
    return h


def _query_with_workspace(lib, h, q, k):
    nq = q.shape[0]
    d = torch.empty(nq, k, device="cuda")
    i = torch.empty(nq, k, dtype=torch.int32, device="cuda")
    ws_bytes = lib.tk_tree_query_workspace_size(h, nq)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
    st = lib.tk_tree_query(h, q.data_ptr(), nq, k, d.data_ptr(), i.data_ptr(), None, ws.data_ptr(), ws_bytes,
                           torch.cuda.current_stream().cuda_stream)
    assert st == 0, lib.tk_last_error()
    return d, i


def _query_noalloc(lib, h, q, k):
    nq = q.shape[0]
    d = torch.full((nq, k), -1.0, device="cuda")
    i = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
    st = lib.tk_tree_query_noalloc(h, q.data_ptr(), nq, k, d.data_ptr(), i.data_ptr(), None,
                                   torch.cuda.current_stream().cuda_stream)
    assert st == 0, lib.tk_last_error()
    return d, i


def test_noalloc_matches_workspace_query_twice():
    from torch_kdtree_gb300._lib import LIB
    rng = np.random.default_rng(2024)
    pts = rng.random((200_000, 3)).astype(np.float32)
    h = _tree(LIB, pts, 14)
    try:
        # two calls in a row with different sizes and k: the second call
        # inherits the first one's scratch contents
        for nq, k in ((150_000, 16), (70_001, 5)):
            q = torch.from_numpy((rng.random((nq, 3)) * 1.2 - 0.1).astype(np.float32)).cuda()
            d_ref, i_ref = _query_with_workspace(LIB, h, q, k)
            d, i = _query_noalloc(LIB, h, q, k)
            torch.cuda.synchronize()
            assert torch.equal(d, d_ref)
            assert torch.equal(i, i_ref)
    finally:
        LIB.tk_tree_destroy(h)


@pytest.mark.parametrize("dims", [2, 5, 8])
def test_noalloc_other_dimensions(dims):
    """Trees of 1-2 and 4-8 dimensions go through the same static scratch."""
    from torch_kdtree_gb300._lib import LIB
    rng = np.random.default_rng(dims)
    pts = rng.standard_normal((50_000, dims)).astype(np.float32)
    h = _tree(LIB, pts, 11)
    try:
        q = torch.from_numpy(rng.standard_normal((40_000, dims)).astype(np.float32)).cuda()
        d_ref, i_ref = _query_with_workspace(LIB, h, q, 12)
        d, i = _query_noalloc(LIB, h, q, 12)
        torch.cuda.synchronize()
        assert torch.equal(d, d_ref)
        assert torch.equal(i, i_ref)
    finally:
        LIB.tk_tree_destroy(h)


def test_noalloc_rejects_oversize_requests():
    from torch_kdtree_gb300._lib import LIB, TK_EINVAL, TK_NOALLOC_MAX_QUERIES
    pts = np.random.default_rng(1).random((1000, 3)).astype(np.float32)
    h = _tree(LIB, pts, 6)
    try:
        nq = TK_NOALLOC_MAX_QUERIES + 1
        q = torch.zeros(nq, 3, device="cuda")
        d = torch.empty(nq, 1, device="cuda")
        i = torch.empty(nq, 1, dtype=torch.int32, device="cuda")
        st = LIB.tk_tree_query_noalloc(h, q.data_ptr(), nq, 1, d.data_ptr(), i.data_ptr(), None,
                                       torch.cuda.current_stream().cuda_stream)
        assert st == TK_EINVAL
        assert "at most" in LIB.tk_last_error().decode()
    finally:
        LIB.tk_tree_destroy(h)
