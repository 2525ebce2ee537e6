"""Autotuner for the KD query launch: tree depth (leaf size), traversal
(per-query stacks or warp packets), lanes per query and node-box pruning.

For a given reference cloud, a query sample and k, it builds the tree at a
few depths around the reference's heuristic, times every lanes-per-query
shape with CUDA events, and keeps the fastest.  Results do not depend on the
choice (the search is exact with a shape-independent tie rule), only speed
does.  Choices are cached in a JSON file keyed by (n, query count bucket, k,
dims, dtype, GPU name).
"""
from __future__ import annotations

import json
import math
import os
from dataclasses import asdict, dataclass
from typing import Optional, Sequence

import torch

from ._lib import QueryOpts
from .nn_distance import TorchKDTree, build_kd_tree, default_levels, knn_query_raw

CACHE_PATH = os.environ.get("TK_AUTOTUNE_CACHE",
                            os.path.join(os.path.expanduser("~"), ".cache", "torch_kdtree_gb300", "autotune.json"))
LANES = (1, 2, 4, 8, 16, 32)


@dataclass
class Choice:
    levels: int
    threads_per_query: int
    ms: float
    plain_levels: int
    table: list  # (levels, lanes, boxes, traversal, ms) of every timed candidate
    prune_boxes: int = 1
    traversal: int = 1  # 1 = per-query stacks, 2 = warp packets

    def opts(self) -> QueryOpts:
        return QueryOpts.make(threads_per_query=self.threads_per_query, prune_boxes=self.prune_boxes,
                              traversal=self.traversal)


def _key(n, nq, k, d, dtype, device) -> str:
    name = torch.cuda.get_device_name(device)
    return f"v2|{name}|n={n}|q~2^{int(round(math.log2(max(nq, 1))))}|k={k}|d={d}|{dtype}"


def _load_cache() -> dict:
    try:
        with open(CACHE_PATH) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store_cache(c: dict) -> None:
    try:
        os.makedirs(os.path.dirname(CACHE_PATH), exist_ok=True)
        with open(CACHE_PATH, "w") as f:
            json.dump(c, f, indent=1)
    except OSError:
        pass


def time_query(tree: TorchKDTree, q: torch.Tensor, k: int, opts: QueryOpts, reps: int = 3) -> float:
    """Median milliseconds of one tk_tree_query (binning + KD kernel)."""
    d = torch.empty(q.shape[0], k, dtype=tree.dtype, device=q.device)
    i = torch.empty(q.shape[0], k, dtype=torch.int32, device=q.device)
    knn_query_raw(tree._tree, q, k, d, i, opts)  # warm-up
    times = []
    for _ in range(reps):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        knn_query_raw(tree._tree, q, k, d, i, opts)
        e.record()
        e.synchronize()
        times.append(s.elapsed_time(e))
    times.sort()
    return times[len(times) // 2]


def autotune(points_ref: torch.Tensor, queries: torch.Tensor, k: int,
             levels_candidates: Optional[Sequence[int]] = None, lanes: Sequence[int] = LANES,
             reps: int = 3, use_cache: bool = True, max_queries: int = 1 << 20) -> Choice:
    """Pick (levels, traversal, threads_per_query, prune_boxes) for querying
    ``points_ref`` with queries like ``queries`` (a sample of at most
    ``max_queries`` is timed)."""
    n, d = points_ref.shape
    key = _key(n, queries.shape[0], k, d, str(points_ref.dtype), points_ref.device)
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        return Choice(**cache[key])
    L0 = default_levels(n)
    if levels_candidates is None:
        # deepest useful tree keeps >= ~4 points per leaf
        lmax = max(1, min(24, int(math.log2(max(n, 2))) - 2))
        levels_candidates = sorted({max(1, min(lmax, L)) for L in range(L0 - 1, L0 + 7)})
    q = queries[:max_queries].contiguous()
    table = []
    best = None
    for L in levels_candidates:
        try:
            tree = build_kd_tree(points_ref, levels=L)
        except Exception:  # too deep for this cloud
            continue
        # a lane holds <= 16 keys; trees of more than 3 dims run 1 or 32 lanes per
        # query and the per-query-stack traversal only
        shapes = [g for g in lanes if g * 16 >= k and (d <= 3 or g in (1, 32))]
        # node-box pruning is an option for trees of 4-8 dims only (1-3 dims always prune with boxes)
        cands = [(g, boxes, 1) for g in shapes for boxes in ((1, 0) if d > 3 else (1,))]
        if k <= 16 and d <= 3:
            cands.append((1, 1, 2))  # warp packets
        for g, boxes, trav in cands:
            ms = time_query(tree, q, k, QueryOpts.make(threads_per_query=g, prune_boxes=boxes, traversal=trav), reps)
            table.append((L, g, boxes, trav, ms))
            if best is None or ms < best[4]:
                best = (L, g, boxes, trav, ms)
        del tree
    ch = Choice(levels=best[0], threads_per_query=best[1], ms=best[4], plain_levels=L0, table=table,
                prune_boxes=best[2], traversal=best[3])
    if use_cache:
        cache[key] = asdict(ch)
        _store_cache(cache)
    return ch


def build_tuned_kd_tree(points_ref: torch.Tensor, queries: torch.Tensor, k: int, **kw) -> TorchKDTree:
    """build_kd_tree with the autotuned depth and launch options."""
    ch = autotune(points_ref, queries, k, **kw)
    return build_kd_tree(points_ref, levels=ch.levels, query_opts=ch.opts())


def autotune_brute(points_ref: torch.Tensor, points_query: torch.Tensor, k: int, reps: int = 3,
                   use_cache: bool = True, max_queries: int = 16384) -> str:
    """Pick the fastest exhaustive-search mode for these shapes: "exact" (CUDA
    cores) or, for float32 with d <= 64 and k <= 64, "tf32" / "bf16_split"
    (tensor-core candidates + exact re-rank).  Every mode returns the same
    exact answer, so only speed decides.  A sample of at most ``max_queries``
    queries is timed; choices are cached like the KD launch choices."""
    from .nn_distance import nn_distance_raw
    n, d = points_ref.shape
    key = "brute|" + _key(n, points_query.shape[0], k, d, str(points_ref.dtype), points_ref.device)
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        return cache[key]["mode"]
    modes = ["exact"]
    if points_ref.dtype == torch.float32 and d <= 64 and k <= 64:
        modes += ["tf32", "bf16_split"]
    q = points_query[:max_queries].contiguous()
    ref = points_ref.contiguous()
    dd = torch.empty(q.shape[0], k, dtype=ref.dtype, device=ref.device)
    ii = torch.empty(q.shape[0], k, dtype=torch.int32, device=ref.device)
    best, table = None, []
    for m in modes:
        nn_distance_raw(ref, q, k, dd, ii, m)  # warm-up
        times = []
        for _ in range(reps):
            s = torch.cuda.Event(enable_timing=True)
            e = torch.cuda.Event(enable_timing=True)
            s.record()
            nn_distance_raw(ref, q, k, dd, ii, m)
            e.record()
            e.synchronize()
            times.append(s.elapsed_time(e))
        ms = sorted(times)[len(times) // 2]
        table.append((m, ms))
        if best is None or ms < best[1]:
            best = (m, ms)
    if use_cache:
        cache[key] = {"mode": best[0], "table": table}
        _store_cache(cache)
    return best[0]
