"""Python API of the engine, mirroring torch_kdtree's (torch_kdtree/nn_distance.py).

    tree = build_kd_tree(points_ref)                 # KD-tree in the reference's layout, on the GPU
    dists, inds = tree.query(points_query, nr_nns_searches=k)

Same names, argument meaning and error behaviour as the reference:
``build_kd_tree(points_ref, device=None, squared_distances=True, levels=None)``
and ``TorchKDTree.query(points_query, nr_nns_searches=1, result_dists=None,
result_idx=None)``.  Differences, all deliberate:

* ``inds`` are int32 original indices computed on the GPU (the reference
  returned ``shuffled_ind[result_idx].long()``, int64); ``inds.long()`` gives
  the reference's dtype.
* among neighbours at exactly equal distance the lower original index wins
  (the reference kept the first one its traversal visited);
* gradients flow through a hand-written, deterministic backward kernel
  instead of torch indexing with atomics;
* ``levels`` may exceed 13 (the reference's limit came from its kernel's
  shared-memory visit tags), up to 24;
* a tree built with ``device='cpu'`` (the reference's KDTreeCPU classes) is
  queried on the host by the library's own threaded search
  (tk_tree_query_cpu), with exactly the GPU query's answers.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Union

import numpy as np
import torch

from . import _lib
from ._lib import LIB, QueryOpts, TreeInfo, check

gpu_available = bool(torch.cuda.is_available() and LIB.tk_cuda_available())

_DTYPES = {torch.float32: _lib.TK_F32, torch.float64: _lib.TK_F64}
MAX_LEVELS = 24
MAX_K = 128
MAX_DIMS = 8  # KD-tree dimensions (1-3 as the reference compiles, 4-8 as its README recipe adds)


def default_levels(n: int) -> int:
    """The reference's heuristic: max(1, min(13, floor(log2 n) - 3))
    (torch_kdtree/nn_distance.py:146-147)."""
    return int(np.maximum(1, np.minimum(13, int(np.log(int(n)) / np.log(2)) - 3)))


def _stream_ptr(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _workspace(nbytes: int, device: torch.device) -> torch.Tensor:
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device)


class _Tree:
    """Owner of a tk_tree handle: built on the host from a numpy array, or
    (``from_device``) on the GPU from a CUDA tensor."""

    def __init__(self, points: Optional[np.ndarray], levels: int, device_index: int):
        self.handle = None
        if points is None:
            return
        n, d = points.shape
        dt = _lib.TK_F32 if points.dtype == np.float32 else _lib.TK_F64
        h = ctypes.c_void_p()
        check(LIB.tk_tree_create(points.ctypes.data, n, d, dt, levels, device_index, 0, ctypes.byref(h)))
        self.handle = h

    @classmethod
    def from_device(cls, points: torch.Tensor, levels: int) -> "_Tree":
        t = cls(None, levels, points.device.index)
        n, d = points.shape
        h = ctypes.c_void_p()
        check(LIB.tk_tree_create_device(points.data_ptr(), n, d, _DTYPES[points.dtype], levels, points.device.index,
                                        _stream_ptr(points.device), ctypes.byref(h)))
        t.handle = h
        return t

    def info(self) -> TreeInfo:
        info = TreeInfo()
        check(LIB.tk_tree_get_info(self.handle, ctypes.byref(info)))
        return info

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            LIB.tk_tree_destroy(h)
            self.handle = None


def knn_query_raw(tree: _Tree, q: torch.Tensor, k: int, dists: torch.Tensor, idx: torch.Tensor,
                  opts: Optional[QueryOpts] = None) -> None:
    """Enqueue one tk_tree_query on the current stream (inputs already on the device)."""
    nq = q.shape[0]
    ws_bytes = LIB.tk_tree_query_workspace_size(tree.handle, nq)
    ws = _workspace(ws_bytes, q.device)
    check(LIB.tk_tree_query(tree.handle, q.data_ptr(), nq, k, dists.data_ptr(), idx.data_ptr(),
                            ctypes.byref(opts) if opts is not None else None, ws.data_ptr(), ws_bytes,
                            _stream_ptr(q.device)))


def knn_query_host(tree: _Tree, q: torch.Tensor, k: int, dists: torch.Tensor, idx: torch.Tensor, device: torch.device,
                   opts: Optional[QueryOpts] = None, transfer: int = _lib.TK_HOST_AUTO) -> None:
    """One tk_tree_query_host: queries and results in host memory; the query
    kernel writes pinned result buffers directly, others are downloaded from
    device staging.  Returns when the results are on the host."""
    check(LIB.tk_tree_query_host(tree.handle, q.data_ptr(), q.shape[0], k, dists.data_ptr(), idx.data_ptr(),
                                 ctypes.byref(opts) if opts is not None else None, int(transfer),
                                 _stream_ptr(device)))


class TorchKDTree:
    def __init__(self, points_ref: torch.Tensor, device: torch.device, levels: int, squared_distances: bool,
                 query_opts: Optional[QueryOpts] = None, build: str = "auto"):
        """Builds the KD-tree.  See :func:`build_kd_tree`."""
        if device.type not in ("cuda", "cpu"):
            raise RuntimeError(f"Could not find the KD-Tree for your specified options (device {device}).")
        if points_ref.shape[0] >= 2 ** 31:
            raise AssertionError("Only 32 bit signed indexing implemented")
        dtype, dims = points_ref.dtype, points_ref.shape[-1]
        if points_ref.dim() != 2 or dtype not in _DTYPES or not 1 <= dims <= MAX_DIMS:
            raise RuntimeError(
                "Could not find the KD-Tree for your specified options. This probably means the library was not "
                f"compiled for the specified dimensionality ({dims}) or precision ({dtype}).")
        if build not in ("auto", "host", "device"):
            raise ValueError("build must be 'auto', 'host' or 'device'")
        if device.type == "cpu":
            # the reference's KDTreeCPU<dims>[F]: built and queried on the host
            if build == "device":
                raise ValueError("a CPU tree is built on the host (build='host' or 'auto')")
            self._setup(points_ref, device, levels, squared_distances, query_opts)
            self.use_gpu = False
            host = np.ascontiguousarray(points_ref.detach().cpu().numpy())
            self._tree = _Tree(host, self.levels, -1)
            self.built_on = "host"
            return
        if device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self._setup(points_ref, device, levels, squared_distances, query_opts)
        if build == "auto":
            build = "device" if points_ref.is_cuda else "host"
        if build == "device":
            pts = points_ref.detach().to(device).contiguous()
            self._tree = _Tree.from_device(pts, self.levels)
        else:
            host = np.ascontiguousarray(points_ref.detach().cpu().numpy())
            self._tree = _Tree(host, self.levels, device.index)
        self.built_on = build

    def _setup(self, points_ref: torch.Tensor, device: torch.device, levels: int, squared_distances: bool,
               query_opts: Optional[QueryOpts]) -> None:
        self.dtype = points_ref.dtype
        self.dims = points_ref.shape[-1]
        self.nr_ref_points = points_ref.shape[0]
        self.device = device
        self.levels = int(levels)
        self.built_on = None
        self.dtype_idx = torch.int32
        self.ref_requires_grad = points_ref.requires_grad
        self.points_ref_bak = points_ref
        self.squared_distances = squared_distances
        self.use_gpu = True
        self.query_opts = query_opts
        self._structured = None
        self._shuffled = None

    def save(self, path) -> None:
        """Write the tree's layout to an ``.npz`` file: the reference's
        ``structured_points`` and ``shuffled_ind`` plus the split values and
        leaf offsets.  :func:`load_kd_tree` re-creates the tree from it
        without rebuilding."""
        np_dtype = np.float32 if self.dtype == torch.float32 else np.float64
        med = np.empty((1 << self.levels) - 1, np_dtype)
        off = np.empty((1 << self.levels) + 1, np.int32)
        check(LIB.tk_tree_get_splits(self._tree.handle, med.ctypes.data, off.ctypes.data))
        perm = np.empty(self.nr_ref_points, np.int32)
        check(LIB.tk_tree_get_perm(self._tree.handle, perm.ctypes.data))
        pts = np.empty((self.nr_ref_points, self.dims), np_dtype)
        check(LIB.tk_tree_get_points(self._tree.handle, pts.ctypes.data))
        np.savez(path, format=np.array(TREE_FORMAT), structured_points=pts, shuffled_ind=perm, split_values=med,
                 leaf_offsets=off, levels=np.int32(self.levels))

    # Layout, as the reference exposes it (torch_kdtree/nn_distance.py:30-41)
    @property
    def structured_points(self) -> torch.Tensor:
        if self._structured is None:
            out = np.empty((self.nr_ref_points, self.dims), dtype=np.float32 if self.dtype == torch.float32
                           else np.float64)
            check(LIB.tk_tree_get_points(self._tree.handle, out.ctypes.data))
            self._structured = torch.from_numpy(out).to(self.device)
        return self._structured

    @property
    def shuffled_ind(self) -> torch.Tensor:
        if self._shuffled is None:
            out = np.empty(self.nr_ref_points, dtype=np.int32)
            check(LIB.tk_tree_get_perm(self._tree.handle, out.ctypes.data))
            self._shuffled = torch.from_numpy(out).long().to(self.device)
        return self._shuffled

    def query(self, points_query: torch.Tensor, nr_nns_searches: int = 1,
              result_dists: Optional[torch.Tensor] = None, result_idx: Optional[torch.Tensor] = None):
        """Exact KNN of ``points_query`` in the tree.

        Returns ``(dists, inds)``: squared (or, with ``squared_distances=False``,
        plain) distances ``[Q, k]`` in the tree's dtype and int32 original
        indices ``[Q, k]``.  Raises RuntimeError when k exceeds the number of
        points, AssertionError on dtype / shape mismatches, as the reference.

        ``result_dists`` / ``result_idx`` may also be CPU tensors (the
        reference takes device buffers only): the results are then written
        there and returned on the CPU.  With CPU queries as well (and no
        gradient), the query is one tk_tree_query_host call: with pinned
        result tensors the query kernel writes them directly."""
        k = int(nr_nns_searches)
        if k > self.nr_ref_points:
            raise RuntimeError("You requested more nearest neighbors than there are in the KD-Tree")
        if k < 1:
            raise RuntimeError("nr_nns_searches must be at least 1")
        if not self.use_gpu:
            return self._query_cpu(points_query, k, result_dists, result_idx)
        if k > MAX_K:
            raise RuntimeError(f"nr_nns_searches is limited to {MAX_K} on the GPU")
        host_out = (result_dists is not None and result_idx is not None and result_dists.device.type == "cpu"
                    and result_idx.device.type == "cpu")
        need_grad = torch.is_grad_enabled() and (points_query.requires_grad or self.ref_requires_grad)
        if host_out and points_query.device.type == "cpu" and not need_grad:
            return self._query_host(points_query, k, result_dists, result_idx)
        out_d = out_i = None
        if host_out:
            self._check_query(points_query, k, result_dists, result_idx)
            out_d, out_i = result_dists, result_idx
            result_dists = result_idx = None
        points_query = points_query.to(self.device)
        nq = points_query.shape[0]
        if result_dists is None:
            result_dists = torch.empty((nq, k), dtype=self.dtype, device=self.device)
        if result_idx is None:
            result_idx = torch.empty((nq, k), dtype=self.dtype_idx, device=self.device)
        self._check_query(points_query, k, result_dists, result_idx)
        if not result_dists.is_contiguous():
            result_dists = result_dists.contiguous()
        if not result_idx.is_contiguous():
            result_idx = result_idx.contiguous()
        if not points_query.is_contiguous():
            points_query = points_query.contiguous()

        need_grad = torch.is_grad_enabled() and (points_query.requires_grad or self.ref_requires_grad)
        if need_grad:
            from .autograd import KnnDistances
            ref = self.points_ref_bak.to(self.device)
            dists, inds = KnnDistances.apply(points_query, ref, self, k)
            with torch.no_grad():
                result_dists.copy_(dists)
                result_idx.copy_(inds)
        else:
            knn_query_raw(self._tree, points_query.detach(), k, result_dists, result_idx, self.query_opts)
            dists, inds = result_dists, result_idx
        if out_d is not None:  # CPU result buffers with device queries or a gradient
            with torch.no_grad():
                out_d.copy_(result_dists)
                out_i.copy_(result_idx)
            dists = out_d if dists is result_dists else dists.to("cpu")
            inds = out_i
        if not self.squared_distances:
            dists = torch.sqrt(dists)
        return dists, inds

    def _check_query(self, points_query: torch.Tensor, k: int, result_dists: torch.Tensor,
                     result_idx: torch.Tensor) -> None:
        nq = points_query.shape[0]
        if list(result_dists.shape) != [nq, k] or result_dists.dtype != self.dtype:
            raise AssertionError("result_dists must be [Q, k] of the tree's dtype")
        if list(result_idx.shape) != [nq, k] or result_idx.dtype != self.dtype_idx:
            raise AssertionError("result_idx must be [Q, k] int32")
        if points_query.dtype != self.dtype:
            raise AssertionError(f"points_query has dtype {points_query.dtype}, the tree {self.dtype}")
        if points_query.dim() != 2 or points_query.shape[1] != self.dims:
            raise AssertionError(f"points_query must be [Q, {self.dims}]")

    def _query_cpu(self, points_query: torch.Tensor, k: int, result_dists: Optional[torch.Tensor],
                   result_idx: Optional[torch.Tensor]):
        """Query of a CPU tree: tk_tree_query_cpu on host memory (the
        reference's KDTreeCPU query, src/kdtree.cpp:164-194).  With a gradient
        the distances are re-gathered by torch, as the reference does
        (torch_kdtree/nn_distance.py:111-112)."""
        points_query = points_query.to(self.device)
        nq = points_query.shape[0]
        if result_dists is None:
            result_dists = torch.empty((nq, k), dtype=self.dtype)
        if result_idx is None:
            result_idx = torch.empty((nq, k), dtype=self.dtype_idx)
        self._check_query(points_query, k, result_dists, result_idx)
        if result_dists.device.type != "cpu" or result_idx.device.type != "cpu":
            raise AssertionError("a CPU tree writes its results into CPU tensors")
        if not result_dists.is_contiguous():
            result_dists = result_dists.contiguous()
        if not result_idx.is_contiguous():
            result_idx = result_idx.contiguous()
        q = points_query.detach().contiguous()
        check(LIB.tk_tree_query_cpu(self._tree.handle, q.data_ptr(), nq, k, result_dists.data_ptr(),
                                    result_idx.data_ptr(), 0))
        dists, inds = result_dists, result_idx
        if (points_query.requires_grad or self.ref_requires_grad) and torch.is_grad_enabled():
            dists = torch.sum((points_query[:, None] - self.points_ref_bak[inds.long()]) ** 2, dim=-1)
        if not self.squared_distances:
            dists = torch.sqrt(dists)
        return dists, inds

    def _query_host(self, points_query: torch.Tensor, k: int, result_dists: torch.Tensor,
                    result_idx: torch.Tensor):
        """CPU queries into CPU result buffers through tk_tree_query_host."""
        self._check_query(points_query, k, result_dists, result_idx)
        q = points_query.detach().contiguous()
        if not result_dists.is_contiguous():
            result_dists = result_dists.contiguous()
        if not result_idx.is_contiguous():
            result_idx = result_idx.contiguous()
        knn_query_host(self._tree, q, k, result_dists, result_idx, self.device, self.query_opts)
        dists = result_dists
        if not self.squared_distances:
            dists = torch.sqrt(dists)
        return dists, result_idx


def build_kd_tree(points_ref: Union[torch.Tensor, np.ndarray], device: Optional[torch.device] = None,
                  squared_distances: bool = True, levels: Optional[int] = None,
                  query_opts: Optional[QueryOpts] = None, build: str = "auto") -> TorchKDTree:
    """Builds the KD-tree for subsequent queries (torch_kdtree/nn_distance.py:119-160).

    The tree has the reference's layout.  On a CUDA ``device`` it lives on
    the GPU; ``build``: "host" builds it on the CPU (as the reference does)
    and uploads it once; "device" builds it on the GPU from the CUDA tensor
    (same layout, no host copy); "auto" (default) picks "device" for CUDA
    input, else "host".  With ``device='cpu'`` (the reference's KDTreeCPU
    trees) it is built and queried on the host.  ``device`` defaults to
    ``points_ref.device``; ``levels`` defaults to the reference's heuristic
    and may range 1..24."""
    if issubclass(type(points_ref), np.ndarray):
        points_ref = torch.from_numpy(points_ref)
    if device is None:
        device = points_ref.device
    if levels is None:
        levels = default_levels(points_ref.shape[0])
    if issubclass(type(device), str):
        device = torch.device(device)
    assert 1 <= levels <= MAX_LEVELS, f"levels must be in [1, {MAX_LEVELS}]"
    assert issubclass(type(points_ref), torch.Tensor)
    assert device.type != "cuda" or gpu_available, "You requested the KD-Tree on the GPU, but no CUDA device is visible"
    assert device.type in ["cuda", "cpu"]
    return TorchKDTree(points_ref, device, levels, squared_distances, query_opts, build)


TREE_FORMAT = "torch_kdtree_gb300.kdtree/1"


def load_kd_tree(path, device: Optional[torch.device] = None, squared_distances: bool = True,
                 query_opts: Optional[QueryOpts] = None) -> TorchKDTree:
    """Re-create a tree written by :meth:`TorchKDTree.save` on ``device``
    (default: the current CUDA device) without rebuilding it.  The layout is
    validated by the library (a corrupt file raises instead of giving inexact
    answers).  Queries and gradients behave as on the saved tree."""
    with np.load(path, allow_pickle=False) as z:
        if str(z["format"]) != TREE_FORMAT:
            raise ValueError(f"{path} is not a {TREE_FORMAT} file")
        pts = np.ascontiguousarray(z["structured_points"])
        perm = np.ascontiguousarray(z["shuffled_ind"], dtype=np.int32)
        med = np.ascontiguousarray(z["split_values"], dtype=pts.dtype)
        off = np.ascontiguousarray(z["leaf_offsets"], dtype=np.int32)
        levels = int(z["levels"])
    if pts.ndim != 2 or pts.dtype not in (np.float32, np.float64):
        raise ValueError("structured_points must be [n, dims] float32 or float64")
    n, d = pts.shape
    if perm.shape != (n,) or med.shape != ((1 << levels) - 1,) or off.shape != ((1 << levels) + 1,):
        raise ValueError("layout arrays have inconsistent shapes")
    device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if device.type not in ("cuda", "cpu"):
        raise RuntimeError(f"trees live on a CUDA device or on the CPU, not {device}")
    if device.type == "cuda" and device.index is None:
        device = torch.device("cuda", torch.cuda.current_device())
    ordinal = device.index if device.type == "cuda" else -1
    h = ctypes.c_void_p()
    check(LIB.tk_tree_create_from_layout(pts.ctypes.data, perm.ctypes.data, med.ctypes.data, off.ctypes.data, n, d,
                                         _lib.TK_F32 if pts.dtype == np.float32 else _lib.TK_F64, levels,
                                         ordinal, ctypes.byref(h)))
    orig = np.empty_like(pts)
    orig[perm] = pts  # the cloud in its original order, for gradients
    tree = TorchKDTree.__new__(TorchKDTree)
    tree._setup(torch.from_numpy(orig).to(device), device, levels, squared_distances, query_opts)
    tree.use_gpu = device.type == "cuda"
    tree._tree = _Tree(None, levels, ordinal)
    tree._tree.handle = h
    tree.built_on = "file"
    return tree


_BRUTE_MODES = {"exact": _lib.TK_BRUTE_EXACT, "fp32": _lib.TK_BRUTE_EXACT, "fp64": _lib.TK_BRUTE_EXACT,
                "tf32": _lib.TK_BRUTE_TF32, "bf16_split": _lib.TK_BRUTE_BF16_SPLIT}


def nn_distance_raw(points_ref: torch.Tensor, points_query: torch.Tensor, k: int, dists: torch.Tensor,
                    idx: torch.Tensor, mode: str = "exact") -> None:
    """Enqueue one tk_nn_distance on the current stream (inputs on the device)."""
    m = _BRUTE_MODES[mode]
    n, d = points_ref.shape
    nq = points_query.shape[0]
    dt = _DTYPES[points_ref.dtype]
    ws_bytes = LIB.tk_nn_distance_workspace_size(n, nq, d, k, dt, m)
    ws = _workspace(ws_bytes, points_ref.device)
    check(LIB.tk_nn_distance(points_ref.data_ptr(), n, points_query.data_ptr(), nq, d, k, dt, m,
                             dists.data_ptr(), idx.data_ptr(), ws.data_ptr(), ws_bytes,
                             _stream_ptr(points_ref.device)))


def nn_distance(points_ref: torch.Tensor, points_query: torch.Tensor, nr_nns_searches: int = 1,
                mode: str = "exact"):
    """Exhaustive exact KNN: ``(dists, inds)`` of every query among all
    reference points, squared distances ``[Q, k]`` and int32 indices.

    ``mode``: "exact" (CUDA cores, float32 or float64), "tf32" or
    "bf16_split" (tensor-core candidate search with an exact float32 re-rank;
    same answer), or "auto" (the fastest of these for the shapes, timed once
    by :func:`torch_kdtree_gb300.autotune.autotune_brute` and cached).
    Differentiable in both point sets.  The reference shipped this search as
    an unbound CUDA launcher (src/nndistance_g.cu:191-220) for d = 3 only;
    here any 1 <= d <= 128, float32 or float64."""
    if mode not in _BRUTE_MODES and mode != "auto":
        raise ValueError(f"mode must be one of {sorted(_BRUTE_MODES) + ['auto']}")
    if points_ref.device.type != "cuda":
        raise RuntimeError("nn_distance runs on CUDA tensors only")
    if points_ref.dtype not in _DTYPES or points_query.dtype != points_ref.dtype:
        raise AssertionError("points must be float32 or float64 and of the same dtype")
    if points_ref.dim() != 2 or points_query.dim() != 2 or points_query.shape[1] != points_ref.shape[1]:
        raise AssertionError("points must be [N, d] and [Q, d]")
    k = int(nr_nns_searches)
    if k > points_ref.shape[0]:
        raise RuntimeError("You requested more nearest neighbors than there are reference points")
    points_query = points_query.to(points_ref.device)
    if mode == "auto":
        from .autotune import autotune_brute
        mode = autotune_brute(points_ref.detach(), points_query.detach(), k)
    ref_c = points_ref.contiguous()
    q_c = points_query.contiguous()
    need_grad = torch.is_grad_enabled() and (points_ref.requires_grad or points_query.requires_grad)
    if need_grad:
        from .autograd import BruteDistances
        return BruteDistances.apply(q_c, ref_c, k, mode)
    nq = q_c.shape[0]
    dists = torch.empty((nq, k), dtype=ref_c.dtype, device=ref_c.device)
    idx = torch.empty((nq, k), dtype=torch.int32, device=ref_c.device)
    nn_distance_raw(ref_c.detach(), q_c.detach(), k, dists, idx, mode)
    return dists, idx


def nn_distance_bidirectional(xyz1: torch.Tensor, xyz2: torch.Tensor, nr_nns_searches: int = 1,
                              mode: str = "exact"):
    """Both directions of the exhaustive search, as the chamfer-style
    NmDistance op computes them: ``(dist1, idx1, dist2, idx2)`` with
    ``dist1, idx1`` the neighbours of every point of ``xyz1`` among ``xyz2``
    and ``dist2, idx2`` those of ``xyz2`` among ``xyz1``.  The reference's
    launcher has the second direction commented out
    (src/nndistance_g.cu:168,219).  Exact and differentiable like
    :func:`nn_distance`; the two searches run back to back on the current
    stream."""
    dist1, idx1 = nn_distance(xyz2, xyz1, nr_nns_searches, mode)
    dist2, idx2 = nn_distance(xyz1, xyz2, nr_nns_searches, mode)
    return dist1, idx1, dist2, idx2
