"""Many point clouds, each with its own tree and its own k, queried in one
persistent launch (tk_batch_* in include/tk_knn.h).

    trees = BatchedKDTrees([ref0, ref1, ...], ks=[1, 16, ...], query_counts=[500, 20, ...])
    dists, inds = trees.query([q0, q1, ...])        # lists of [Q_c, k_c] tensors
    replay = trees.graph(q_flat)                     # CUDA graph of the whole batched query
    replay()                                         # -> trees.out_dists / trees.out_idx (flat)

The reference queried one cloud per call; this is the batched pattern of the
engine, equivalent bit for bit to querying every tree on its own.  Trees of
1-8 dimensions (one dims per batch).
"""
from __future__ import annotations

import ctypes
from typing import List, Optional, Sequence

import torch

from ._lib import LIB, QueryOpts, check
from .nn_distance import TorchKDTree, _stream_ptr, _workspace, build_kd_tree, knn_query_raw


class BatchedKDTrees:
    def __init__(self, clouds: Sequence[torch.Tensor], ks: Sequence[int], query_counts: Sequence[int],
                 levels: Optional[Sequence[Optional[int]]] = None, device: Optional[torch.device] = None,
                 threads_per_query: int = 0, prune_boxes: bool = False):
        if not (len(clouds) == len(ks) == len(query_counts)) or not clouds:
            raise ValueError("clouds, ks and query_counts must be non-empty and of equal length")
        device = torch.device(device) if device is not None else clouds[0].device
        if device.type != "cuda":
            raise RuntimeError("batched trees live on a CUDA device")
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        levels = list(levels) if levels is not None else [None] * len(clouds)
        self.device = device
        self.trees: List[TorchKDTree] = [build_kd_tree(c, device=device, levels=L) for c, L in zip(clouds, levels)]
        self.ks = [int(k) for k in ks]
        self.query_counts = [int(n) for n in query_counts]
        self.dtype = self.trees[0].dtype
        self.dims = self.trees[0].dims
        self.threads_per_query = int(threads_per_query)
        self.prune_boxes = int(bool(prune_boxes))
        handles = (ctypes.c_void_p * len(self.trees))(*[t._tree.handle.value for t in self.trees])
        qc = (ctypes.c_int64 * len(self.trees))(*self.query_counts)
        kk = (ctypes.c_int32 * len(self.trees))(*self.ks)
        h = ctypes.c_void_p()
        check(LIB.tk_batch_create(handles, len(self.trees), qc, kk, ctypes.byref(h)))
        self._h = h
        self.total_queries = sum(self.query_counts)
        self.total_out = int(LIB.tk_batch_output_size(h))
        self.ws_bytes = int(LIB.tk_batch_workspace_size(h))
        self._ws = _workspace(self.ws_bytes, device)
        self.out_dists = torch.empty(self.total_out, dtype=self.dtype, device=device)
        self.out_idx = torch.empty(self.total_out, dtype=torch.int32, device=device)
        offs, o = [], 0
        for n, k in zip(self.query_counts, self.ks):
            offs.append(o)
            o += n * k
        self._out_offsets = offs

    def query_flat(self, q_flat: torch.Tensor, out_dists: Optional[torch.Tensor] = None,
                   out_idx: Optional[torch.Tensor] = None) -> None:
        """Enqueue the batched query of concatenated queries ``q_flat``
        ``[sum Q_c, d]``; results go to ``out_dists`` / ``out_idx`` (flat,
        cloud c's ``[Q_c, k_c]`` block after cloud c-1's)."""
        out_dists = self.out_dists if out_dists is None else out_dists
        out_idx = self.out_idx if out_idx is None else out_idx
        if q_flat.shape != (self.total_queries, self.dims) or q_flat.dtype != self.dtype:
            raise AssertionError(f"queries must be [{self.total_queries}, {self.dims}] {self.dtype}")
        if not q_flat.is_contiguous() or q_flat.device != self.device:
            raise AssertionError("queries must be contiguous on the batch's device")
        check(LIB.tk_batch_query(self._h, q_flat.data_ptr(), out_dists.data_ptr(), out_idx.data_ptr(),
                                 self.threads_per_query, self.prune_boxes, self._ws.data_ptr(), self.ws_bytes,
                                 _stream_ptr(self.device)))

    def split(self, flat: torch.Tensor) -> List[torch.Tensor]:
        return [flat[o:o + n * k].view(n, k) for o, n, k in zip(self._out_offsets, self.query_counts, self.ks)]

    def query(self, queries: Sequence[torch.Tensor]):
        """Batched query of per-cloud query tensors; returns lists of
        ``[Q_c, k_c]`` distances and int32 indices."""
        if len(queries) != len(self.trees):
            raise ValueError("one query tensor per cloud")
        for q, n in zip(queries, self.query_counts):
            if q.shape[0] != n:
                raise AssertionError("query counts differ from the batch plan")
        q_flat = torch.cat([q.to(self.device, self.dtype) for q in queries]).contiguous()
        d = torch.empty(self.total_out, dtype=self.dtype, device=self.device)
        i = torch.empty(self.total_out, dtype=torch.int32, device=self.device)
        self.query_flat(q_flat, d, i)
        return self.split(d), self.split(i)

    def query_each(self, queries: Sequence[torch.Tensor], out_dists: Optional[torch.Tensor] = None,
                   out_idx: Optional[torch.Tensor] = None, opts: Optional[QueryOpts] = None) -> None:
        """The same work as one launch per cloud (tk_tree_query per tree),
        writing into the flat outputs -- the baseline the batch replaces."""
        out_dists = self.out_dists if out_dists is None else out_dists
        out_idx = self.out_idx if out_idx is None else out_idx
        ds, is_ = self.split(out_dists), self.split(out_idx)
        for t, q, k, d, i in zip(self.trees, queries, self.ks, ds, is_):
            if q.shape[0]:
                knn_query_raw(t._tree, q, k, d, i, opts)

    def graph(self, q_flat: torch.Tensor):
        """Capture the batched query of ``q_flat`` in a CUDA graph; returns a
        function that replays it (results in ``out_dists`` / ``out_idx``)."""
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.query_flat(q_flat)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.query_flat(q_flat)
        self._graph = g
        return g.replay

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            LIB.tk_batch_destroy(h)
            self._h = None
