"""ORACLE -- test infrastructure, not part of the product.

ctypes front end for the oracle libraries built by ``oracle/Makefile``:

* ``liboracle.so`` -- our plain-C restatement of the reference's CPU KD-tree
  (build: src/kdtree.hpp:392-534; query: src/kdtree.cpp:16-110,164-194) and
  an exhaustive search with the same distance arithmetic.
* ``_ref/libtkref.so`` -- the reference's own CPU sources behind a small C
  wrapper (only where the reference checkout was present at build time).

Plus numpy helpers: FP64 recomputation of distances, an FP64 brute force for
any dimension, and the tie-aware comparison used by the parity tests.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_REF = None

_c_i32p = ctypes.POINTER(ctypes.c_int32)
_c_u8p = ctypes.POINTER(ctypes.c_uint8)


def build(ref: bool | str = False) -> None:
    """Compile liboracle.so and, with ref=True, the reference's own CPU
    sources (oracle/_ref); ref="if-present" builds the latter only where the
    Makefile's REF_SRC (environment variable TK_REFERENCE_SRC) holds them."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref == "if-present":
        subprocess.run(["make", "-s", "-C", HERE, "ref-if-present"], check=True)
    elif ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        for sfx in ("f32", "f64"):
            getattr(L, f"orc_build_{sfx}").restype = ctypes.c_int
            getattr(L, f"orc_query_{sfx}").restype = ctypes.c_int
            getattr(L, f"orc_brute_{sfx}").restype = ctypes.c_int
        _LIB = L
    return _LIB


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libtkref.so"))


def ref_lib():
    global _REF
    if _REF is None:
        L = ctypes.CDLL(os.path.join(HERE, "_ref", "libtkref.so"))
        L.ref_tree_create.restype = ctypes.c_void_p
        L.ref_tree_create.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.ref_tree_layout.argtypes = [ctypes.c_void_p] * 7
        L.ref_tree_query.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int,
                                     ctypes.c_void_p, ctypes.c_void_p]
        L.ref_tree_destroy.argtypes = [ctypes.c_void_p]
        L.ref_last_error.restype = ctypes.c_char_p
        _REF = L
    return _REF


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _sfx(dtype) -> str:
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f32"
    if dt == np.float64:
        return "f64"
    raise TypeError(f"unsupported dtype {dt}")


def default_levels(n: int) -> int:
    """build_kd_tree's heuristic (torch_kdtree/nn_distance.py:146-147)."""
    return int(max(1, min(13, int(np.log(int(n)) / np.log(2)) - 3)))


@dataclass
class Layout:
    """A KD-tree in the reference's layout (src/kdtree.hpp:126-217)."""

    levels: int
    structured: np.ndarray  # [n, d] points in leaf order
    perm: np.ndarray        # [n] int32 shuffled_inds: structured[i] == points[perm[i]]
    medians: np.ndarray     # [2^L - 1] split values, heap order
    axes: np.ndarray        # [2^L - 1] uint8 split axes
    leaf_off: np.ndarray    # [2^L] int32
    leaf_cnt: np.ndarray    # [2^L] int32

    @property
    def dims(self) -> int:
        return self.structured.shape[1]


def _alloc_layout(n, d, levels, dtype):
    nparts = (1 << levels) - 1
    return Layout(levels, np.empty((n, d), dtype), np.empty(n, np.int32), np.empty(nparts, dtype),
                  np.empty(nparts, np.uint8), np.empty(nparts + 1, np.int32), np.empty(nparts + 1, np.int32))


def build_tree(points: np.ndarray, levels: int | None = None, nthreads: int = 0) -> Layout:
    """Oracle restatement of createKDTree."""
    points = np.ascontiguousarray(points)
    n, d = points.shape
    if levels is None:
        levels = default_levels(n)
    lay = _alloc_layout(n, d, levels, points.dtype)
    nthreads = nthreads or os.cpu_count() or 1
    rc = getattr(lib(), f"orc_build_{_sfx(points.dtype)}")(
        _ptr(points), ctypes.c_int32(n), ctypes.c_int(d), ctypes.c_int(levels), _ptr(lay.structured),
        _ptr(lay.perm), _ptr(lay.medians), _ptr(lay.axes), _ptr(lay.leaf_off), _ptr(lay.leaf_cnt),
        ctypes.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle build failed ({rc}): ran out of points or bad arguments")
    return lay


def query_tree(lay: Layout, q: np.ndarray, k: int, nthreads: int = 0, local: bool = False):
    """Oracle restatement of KDTreeKNNSearch.  Returns (dists, idx); idx are
    original indices unless ``local`` (structured order, as the C++ returns)."""
    q = np.ascontiguousarray(q, dtype=lay.structured.dtype)
    nq = q.shape[0]
    dists = np.empty((nq, k), lay.structured.dtype)
    idx = np.empty((nq, k), np.int32)
    nthreads = nthreads or os.cpu_count() or 1
    rc = getattr(lib(), f"orc_query_{_sfx(q.dtype)}")(
        _ptr(lay.structured), ctypes.c_int(lay.dims), ctypes.c_int(lay.levels), _ptr(lay.medians),
        _ptr(lay.axes), _ptr(lay.leaf_off), _ptr(lay.leaf_cnt), _ptr(q), ctypes.c_int64(nq),
        ctypes.c_int(k), _ptr(dists), _ptr(idx), ctypes.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle query failed ({rc})")
    if not local:
        idx = lay.perm[idx]
    return dists, idx


def brute(ref: np.ndarray, q: np.ndarray, k: int, nthreads: int = 0):
    """Exhaustive k smallest (distance, original index) with the reference's
    distance arithmetic.  The canonical answer of every GPU path."""
    ref = np.ascontiguousarray(ref)
    q = np.ascontiguousarray(q, dtype=ref.dtype)
    n, d = ref.shape
    nq = q.shape[0]
    dists = np.empty((nq, k), ref.dtype)
    idx = np.empty((nq, k), np.int32)
    nthreads = nthreads or os.cpu_count() or 1
    rc = getattr(lib(), f"orc_brute_{_sfx(ref.dtype)}")(
        _ptr(ref), ctypes.c_int64(n), _ptr(q), ctypes.c_int64(nq), ctypes.c_int(d), ctypes.c_int(k),
        _ptr(dists), _ptr(idx), ctypes.c_int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle brute force failed ({rc})")
    return dists, idx


# ------------------------------------------------- the reference itself --

class RefTree:
    """The reference's own CPU KD-tree (compiled from its sources)."""

    def __init__(self, points: np.ndarray, levels: int | None = None):
        self.points = np.ascontiguousarray(points)
        n, d = self.points.shape
        self.levels = default_levels(n) if levels is None else levels
        dt = 0 if self.points.dtype == np.float32 else 1
        self._h = ref_lib().ref_tree_create(_ptr(self.points), n, d, dt, self.levels)
        if not self._h:
            raise RuntimeError(ref_lib().ref_last_error().decode())

    def layout(self) -> Layout:
        n, d = self.points.shape
        lay = _alloc_layout(n, d, self.levels, self.points.dtype)
        ref_lib().ref_tree_layout(self._h, _ptr(lay.structured), _ptr(lay.perm), _ptr(lay.medians),
                                  _ptr(lay.axes), _ptr(lay.leaf_off), _ptr(lay.leaf_cnt))
        lay.leaf_off = lay.leaf_off[: 1 << self.levels]
        lay.leaf_cnt = lay.leaf_cnt[: 1 << self.levels]
        return lay

    def query(self, q: np.ndarray, k: int, local: bool = False):
        q = np.ascontiguousarray(q, dtype=self.points.dtype)
        nq = q.shape[0]
        dists = np.empty((nq, k), self.points.dtype)
        idx = np.empty((nq, k), np.int32)
        ref_lib().ref_tree_query(self._h, _ptr(q), nq, k, _ptr(dists), _ptr(idx))
        if not local:
            idx = self.layout().perm[idx]
        return dists, idx

    def __del__(self):
        if getattr(self, "_h", None):
            ref_lib().ref_tree_destroy(self._h)
            self._h = None


# ------------------------------------------------------- numpy helpers --

def recompute_f64(ref: np.ndarray, q: np.ndarray, idx: np.ndarray) -> np.ndarray:
    """FP64 squared distances of the returned pairs from the original inputs."""
    r = ref.astype(np.float64)[idx]
    return ((q.astype(np.float64)[:, None, :] - r) ** 2).sum(-1)


def brute_f64(ref: np.ndarray, q: np.ndarray, k: int, chunk: int = 256):
    """FP64 brute force for any dimension: k smallest by (dist64, index)."""
    r64 = ref.astype(np.float64)
    rn = (r64 ** 2).sum(1)
    out_d = np.empty((q.shape[0], k), np.float64)
    out_i = np.empty((q.shape[0], k), np.int64)
    for s in range(0, q.shape[0], chunk):
        qq = q[s:s + chunk].astype(np.float64)
        # exact-difference form for the final ranking of the shortlisted set
        approx = (qq ** 2).sum(1)[:, None] - 2.0 * qq @ r64.T + rn[None, :]
        m = min(ref.shape[0], k + 64)
        cand = np.argpartition(approx, m - 1, axis=1)[:, :m]
        d = ((qq[:, None, :] - r64[cand]) ** 2).sum(-1)
        for row in range(qq.shape[0]):
            o = np.lexsort((cand[row], d[row]))[:k]
            out_d[s + row] = d[row, o]
            out_i[s + row] = cand[row, o]
    return out_d, out_i


@dataclass
class Compare:
    n_queries: int
    mismatches: int        # positions whose index differs and is not explained by a tie
    tie_queries: int       # queries whose lists differ only inside exact-distance ties
    dist_bit_mismatch: int # positions whose distances differ bitwise

    @property
    def ok(self) -> bool:
        return self.mismatches == 0 and self.dist_bit_mismatch == 0


def compare_knn(d_a, i_a, d_b, i_b) -> Compare:
    """Tie-aware comparison of two KNN results over the same inputs.

    Distances must agree bitwise.  Indices may differ only between entries of
    equal distance: within each group of equal distance the index sets must
    match, except for the group holding the k-th distance, which may extend
    past the list (a tie at the boundary)."""
    d_a = np.asarray(d_a)
    d_b = np.asarray(d_b)
    i_a = np.asarray(i_a)
    i_b = np.asarray(i_b)
    bitdiff = int((d_a.view(np.uint8).reshape(d_a.shape + (-1,)) !=
                   d_b.view(np.uint8).reshape(d_b.shape + (-1,))).any(-1).sum())
    rows = np.nonzero((i_a != i_b).any(1))[0]
    mism = 0
    ties = 0
    for r in rows:
        da, ia, ib = d_a[r], i_a[r], i_b[r]
        kth = da[-1]
        bad = 0
        for v in np.unique(da):
            sa = set(ia[da == v].tolist())
            sb = set(ib[d_b[r] == v].tolist())
            if sa != sb and v != kth:
                bad += len(sa ^ sb)
        if bad:
            mism += bad
        else:
            ties += 1
    return Compare(d_a.shape[0], mism, ties, bitdiff)
