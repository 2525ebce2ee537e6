"""autograd.Function wrappers: forward through the KNN kernels, backward
through the deterministic tk_knn_backward kernel (include/tk_knn.h)."""
from __future__ import annotations

import torch

from . import _lib
from ._lib import LIB, check

_DT = {torch.float32: _lib.TK_F32, torch.float64: _lib.TK_F64}


def knn_backward(q: torch.Tensor, ref: torch.Tensor, idx: torch.Tensor, grad_dists: torch.Tensor,
                 need_q: bool = True, need_ref: bool = True):
    """(grad_q, grad_ref) of squared distances for the neighbour list ``idx``."""
    q = q.detach().contiguous()
    ref = ref.detach().contiguous()
    idx = idx.contiguous()
    g = grad_dists.detach().to(q.dtype).contiguous()
    nq, d = q.shape
    n = ref.shape[0]
    k = idx.shape[1]
    gq = torch.empty_like(q) if need_q else None
    gr = torch.empty_like(ref) if need_ref else None
    ws_bytes = LIB.tk_knn_backward_workspace_size(nq, k, n) if need_ref else 0
    ws = torch.empty(max(ws_bytes, 1), dtype=torch.uint8, device=q.device)
    stream = torch.cuda.current_stream(q.device).cuda_stream
    check(LIB.tk_knn_backward(q.data_ptr(), ref.data_ptr(), idx.data_ptr(), g.data_ptr(), nq, n, k, d,
                              _DT[q.dtype], gq.data_ptr() if gq is not None else None,
                              gr.data_ptr() if gr is not None else None, ws.data_ptr(), ws_bytes, stream))
    return gq, gr


class KnnDistances(torch.autograd.Function):
    """dists, inds = KnnDistances.apply(q, ref, tree, k)

    ``ref`` is the original (unpermuted) reference tensor the tree was built
    from; the forward runs the tree query, the backward recomputes the
    differences from the saved indices."""

    @staticmethod
    def forward(ctx, q, ref, tree, k):
        from .nn_distance import knn_query_raw
        result_dists = torch.empty((q.shape[0], k), dtype=q.dtype, device=q.device)
        result_idx = torch.empty((q.shape[0], k), dtype=torch.int32, device=q.device)
        knn_query_raw(tree._tree, q.detach(), k, result_dists, result_idx, tree.query_opts)
        ctx.save_for_backward(q, ref, result_idx)
        ctx.mark_non_differentiable(result_idx)
        return result_dists, result_idx

    @staticmethod
    def backward(ctx, grad_dists, _grad_idx):
        q, ref, idx = ctx.saved_tensors
        need_q, need_ref = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (need_q or need_ref):
            return None, None, None, None
        gq, gr = knn_backward(q, ref, idx, grad_dists, need_q, need_ref)
        return gq, gr, None, None


class BruteDistances(torch.autograd.Function):
    """dists, inds = BruteDistances.apply(q, ref, k, mode): exhaustive search
    forward, same deterministic backward as the tree query."""

    @staticmethod
    def forward(ctx, q, ref, k, mode):
        from .nn_distance import nn_distance_raw
        d = torch.empty((q.shape[0], k), dtype=q.dtype, device=q.device)
        i = torch.empty((q.shape[0], k), dtype=torch.int32, device=q.device)
        nn_distance_raw(ref.detach(), q.detach(), k, d, i, mode)
        ctx.save_for_backward(q, ref, i)
        ctx.mark_non_differentiable(i)
        return d, i

    @staticmethod
    def backward(ctx, grad_dists, _grad_idx):
        q, ref, idx = ctx.saved_tensors
        need_q, need_ref = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        if not (need_q or need_ref):
            return None, None, None, None
        gq, gr = knn_backward(q, ref, idx, grad_dists, need_q, need_ref)
        return gq, gr, None, None
