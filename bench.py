"""Benchmark of the KD-tree KNN query on one GB300.

Workload (default): large single-cloud query, d=3, float32 -- 4,194,304
reference points (half uniform cube, half noisy unit sphere), 1,048,576
queries uniform in [-0.1, 1.1]^3, k = 16.  A step is one exact KNN query of
all queries.  "plain" = the reference's default tree depth and the default
launch shape; "chosen" = autotuned depth and lanes per query, replayed as a
captured CUDA graph.  `value` is the chosen queries/s with inputs resident in
HBM; `e2e` goes through the public API with host buffers.

    python bench.py [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "KNN queries/s (d=3,k=16,4M ref) chosen vs plain on 1 GB300 at exact indices"
UNIT = "queries/s"
K_NN = 16
WORKLOAD = ("large single-cloud KD query: 4,194,304 refs (half U[0,1]^3, half unit sphere at (0.5,0.5,0.5) "
            "with N(0,0.01) radial noise), 1,048,576 queries U[-0.1,1.1]^3, k=16, float32")
L2_FLUSH_BYTES = 512 << 20


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


# ------------------------------------------------------------ clocks --

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, ValueError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------ helpers --

def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback"


def fp64_error(ref, q, dists, idx, chunk=1 << 18):
    """Max relative error of the returned FP32 squared distances against the
    same (query, neighbour) pairs recomputed in FP64 from the FP32 inputs, and
    the number of queries with an exact distance tie inside their returned
    list (ties are ordered by lower original index)."""
    import torch
    worst = 0.0
    ties = 0
    for a in range(0, q.shape[0], chunk):
        qq = q[a:a + chunk].double()
        ii = idx[a:a + chunk].long()
        d64 = ((ref[ii].double() - qq[:, None, :]) ** 2).sum(-1)
        dd = dists[a:a + chunk].double()
        rel = (dd - d64).abs() / d64.clamp_min(torch.finfo(torch.float64).tiny)
        rel = torch.where(d64 > 0, rel, (dd - d64).abs())
        worst = max(worst, float(rel.max()))
        ties += int((dists[a:a + chunk, 1:] == dists[a:a + chunk, :-1]).any(1).sum())
    return {"max_rel_err": worst, "queries_with_equal_distances_in_list": ties}


def profiled_value(kernel_tag: str, field: str = "traffic_bytes_per_launch", shape: str | None = None):
    """A per-launch figure of a kernel from its committed ncu summary
    (profiles/<kernel_tag>.md, line '<field>: <int>'), or None.  With
    `shape`, only if the summary's 'profiled_shape:' line names that launch
    shape (a figure of another shape is not this launch's)."""
    path = os.path.join(ROOT, "profiles", kernel_tag + ".md")
    try:
        text = open(path).read()
    except OSError:
        return None
    if shape is not None:
        m = re.search(r"profiled_shape:\s*(.+)", text)
        if not m or m.group(1).strip() != shape:
            return None
    m = re.search(field + r":\s*([0-9]+)", text)
    return int(m.group(1)) if m else None


def profiled_traffic(kernel_tag: str, shape: str | None = None):
    """DRAM bytes (read + write) per launch from the kernel's ncu summary, or None."""
    return profiled_value(kernel_tag, "traffic_bytes_per_launch", shape)


def launch_shape(levels: int, lanes: int, traversal: int) -> str:
    """The key a profile summary's 'profiled_shape:' line must carry."""
    return f"levels={levels} threads_per_query={lanes} traversal={traversal}"


def issue_roofline(kernel_tag: str, kernel_ms: float, dev_index: int, shape: str | None = None):
    """Instruction-issue roofline of an issue-bound kernel: warp instructions
    per launch (from its ncu summary, of the same launch shape) over the
    measured launch time, against one warp instruction per cycle per
    scheduler (4 per SM) at the maximum SM clock."""
    import torch
    inst = profiled_value(kernel_tag, "warp_instructions_per_launch", shape)
    if inst is None:
        return None
    props = torch.cuda.get_device_properties(dev_index)
    mhz = 2070.0
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    except (OSError, ValueError):
        pass
    peak = props.multi_processor_count * 4 * mhz * 1e6 / 1e9  # G warp instructions / s
    achieved = inst / (kernel_ms / 1e3) / 1e9
    return {"achieved": achieved, "peak": peak, "unit": "G warp instructions/s", "frac": achieved / peak,
            "warp_instructions_per_launch": inst}


def algorithmic_bytes(n_ref, nq, k, levels, d=3):
    """Bytes a KD query launch must move at minimum: queries in (4d per
    query), results out (8k per query: distance + index), and the tree once:
    4d bytes per reference point and 8 bytes per split node (the reference's
    {axis, value} record)."""
    return nq * (4 * d + 8 * k) + 4 * d * n_ref + 8 * ((1 << levels) - 1)


def layout_bytes(n_ref, nq, k, levels, d=3):
    """The same minimum in this engine's layout: 16-byte point records
    (coordinates + original index), 4-byte split values and leaf offsets."""
    return nq * (4 * d + 8 * k) + 16 * n_ref + 4 * ((1 << levels) - 1) + 4 * ((1 << levels) + 1)


# -------------------------------------------------------- reference arm --

def synthetic_module():
    """torch_kdtree_gb300/synthetic.py (pure numpy), loaded by its file path:
    importing it through the package would also load the package's CUDA
    library, which the reference arm must never map."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "tk_synthetic_standalone", os.path.join(ROOT, "torch_kdtree_gb300", "synthetic.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_reference(args):
    """The reference's CPU query path timed on this host's cores: the
    reference's own sources (oracle/_ref) where they were built, else the
    oracle's C restatement of them.  Loads nothing of this package but its
    numpy input generators (by file path), so no library of ours is mapped."""
    from oracle import oracle as O
    O.build()
    ref, q = synthetic_module().cube_and_sphere()
    threads = os.cpu_count() or 1
    kind = "port"
    if O.ref_available():
        try:
            O.ref_lib()
            kind = "reference"
        except OSError:
            kind = "port"
    sample = min(len(q), args.ref_sample)
    qs = q[:sample]
    t0 = time.perf_counter()
    if kind == "reference":
        os.environ["OMP_NUM_THREADS"] = str(threads)
        tree = O.RefTree(ref, O.default_levels(len(ref)))
    else:
        lay = O.build_tree(ref, O.default_levels(len(ref)), nthreads=threads)
    build_s = time.perf_counter() - t0
    times = []
    for step in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        if kind == "reference":
            tree.query(qs, K_NN, local=True)
        else:
            O.query_tree(lay, qs, K_NN, nthreads=threads, local=True)
        dt = time.perf_counter() - t0
        if step >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = sample * len(times) / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy, shapes and distributions of the workload)",
        "config": {"workload": WORKLOAD, "levels": O.default_levels(len(ref)),
                   "sample_queries_per_step": sample, "tree_build_s": build_s,
                   "vs_our_arm": "same cloud, queries and k; the CPU path runs the reference's default depth "
                                 "and times a bounded query sample per step (queries/s is per query), while "
                                 "our arm runs its autotuned depth over all 1,048,576 queries"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"first {sample} of the 1,048,576 queries per step, full 4,194,304-point tree"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- our arm --

def run_ours(args, rank, world):
    import torch

    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300._lib import QueryOpts
    from torch_kdtree_gb300.autotune import autotune
    from torch_kdtree_gb300.nn_distance import knn_query_raw
    from torch_kdtree_gb300.synthetic import cube_and_sphere

    dev = torch.device("cuda", env_int("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    ref_np, q_np = cube_and_sphere(seed=0)
    if rank:  # replicas: same cloud, own queries
        _, q_np = cube_and_sphere(seed=1000 + rank)
    n_ref, nq = ref_np.shape[0], q_np.shape[0]
    ref = torch.from_numpy(ref_np).to(dev)
    q = torch.from_numpy(q_np).to(dev)

    # ---- plain: reference heuristic depth, default launch shape, built on the host like the reference
    t0 = time.perf_counter()
    plain = tk.build_kd_tree(ref, build="host")
    build_plain_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    del_me = tk.build_kd_tree(ref, build="device", levels=plain.levels)
    torch.cuda.synchronize()
    build_plain_dev_s = time.perf_counter() - t0
    del del_me
    # ---- chosen: autotuned depth and lanes per query (or given on the command line)
    t0 = time.perf_counter()
    if args.levels and args.tpq:
        from torch_kdtree_gb300.autotune import Choice
        ch = Choice(levels=args.levels, threads_per_query=args.tpq, ms=float("nan"), plain_levels=plain.levels,
                    table=[], prune_boxes=args.boxes, traversal=args.traversal)
    else:
        ch = autotune(ref, q, K_NN, use_cache=False)
    tune_s = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    chosen = tk.build_kd_tree(ref, levels=ch.levels, query_opts=ch.opts(), build="device")
    torch.cuda.synchronize()
    build_chosen_s = time.perf_counter() - t0

    if args.profile:
        # one query of each tree, nothing else (for ncu captures)
        for tree in (chosen, plain):
            dd = torch.empty(nq, K_NN, device=dev)
            ii = torch.empty(nq, K_NN, dtype=torch.int32, device=dev)
            knn_query_raw(tree._tree, q, K_NN, dd, ii, tree.query_opts)
        torch.cuda.synchronize()
        return

    d_plain = torch.empty(nq, K_NN, device=dev)
    i_plain = torch.empty(nq, K_NN, dtype=torch.int32, device=dev)
    d_ch = torch.empty_like(d_plain)
    i_ch = torch.empty_like(i_plain)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    # chosen step as one captured graph (binning + KD kernel, no host work)
    s = torch.cuda.Stream(dev)
    s.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(s):
        knn_query_raw(chosen._tree, q, K_NN, d_ch, i_ch, chosen.query_opts)
    torch.cuda.current_stream(dev).wait_stream(s)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        knn_query_raw(chosen._tree, q, K_NN, d_ch, i_ch, chosen.query_opts)

    def step_chosen():
        graph.replay()

    def step_plain():
        knn_query_raw(plain._tree, q, K_NN, d_plain, i_plain, plain.query_opts)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            flush.zero_()
            fn()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ms = []
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            b.synchronize()
            ms.append(a.elapsed_time(b))
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return ms

    with ClockSampler(dev.index) as clk:
        ms_chosen = timed(step_chosen, args.steps, args.warmup)
        ms_plain = timed(step_plain, args.steps, args.warmup)
    clocks = clk.summary()

    same = bool(torch.equal(i_plain, i_ch) and torch.equal(d_plain, d_ch))

    # ---- dominant kernel alone (events recorded inside the library around the KD kernel)
    ks = torch.cuda.Event(enable_timing=True)
    ke = torch.cuda.Event(enable_timing=True)
    ks.record()
    ke.record()  # materialise the events
    torch.cuda.synchronize()
    kopts = QueryOpts.make(threads_per_query=ch.threads_per_query, kernel_start_event=ks.cuda_event,
                           kernel_stop_event=ke.cuda_event, prune_boxes=ch.prune_boxes, traversal=ch.traversal)
    kern_ms = []
    for _ in range(max(3, args.steps)):
        flush.zero_()
        knn_query_raw(chosen._tree, q, K_NN, d_ch, i_ch, kopts)
        ke.synchronize()
        kern_ms.append(ks.elapsed_time(ke))
    kern_avg = sum(kern_ms) / len(kern_ms)

    # ---- end to end through the public API, host buffers in and out
    q_host = torch.from_numpy(q_np).pin_memory()
    d_host = torch.empty(nq, K_NN).pin_memory()
    i_host = torch.empty(nq, K_NN, dtype=torch.int32).pin_memory()

    def step_e2e():  # one host-buffer query (tk_tree_query_host): copies pipelined with the search
        chosen.query(q_host, nr_nns_searches=K_NN, result_dists=d_host, result_idx=i_host)

    ms_e2e = timed(step_e2e, args.steps, args.warmup)

    # max over ranks (the slowest replica sets the job time)
    from torch_kdtree_gb300.distributed import world_max
    t_chosen = world_max(sum(ms_chosen), dev)
    t_plain = world_max(sum(ms_plain), dev)
    t_e2e = world_max(sum(ms_e2e), dev)
    if rank != 0:
        return

    value = world * nq * args.steps / (t_chosen / 1e3)
    plain_value = world * nq * args.steps / (t_plain / 1e3)
    peak, peak_kind = measured_peak_hbm()
    alg = algorithmic_bytes(n_ref, nq, K_NN, ch.levels)
    achieved = alg / (kern_avg / 1e3) / 1e9
    kernel_name = "k_kd_packet" if ch.traversal == 2 else "k_kd_query"
    shape = launch_shape(ch.levels, ch.threads_per_query, ch.traversal)
    prof_tag = kernel_name[2:] + "_cube_sphere_4M_k16"
    traffic = profiled_traffic(prof_tag, shape)
    issue = issue_roofline(prof_tag, kern_avg, dev.index, shape)
    fp64 = fp64_error(ref, q, d_ch, i_ch)

    # ---- CPU baseline (oracle / reference CPU path) on a bounded sample, plus an exactness check of that sample
    cpu = None
    exact = None
    if not args.no_cpu_baseline:
        cpu, exact = cpu_baseline(ref_np, q_np, i_ch[: args.ref_sample].cpu().numpy(),
                                  d_ch[: args.ref_sample].cpu().numpy(), args.ref_sample)
    rows = None
    if world == 1 and not args.no_rows:
        rows = run_rows(args, dev, flush)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_chosen / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy, shapes and distributions of the workload)",
        "config": {"workload": WORKLOAD, "levels": ch.levels, "threads_per_query": ch.threads_per_query,
                   "prune_boxes": ch.prune_boxes, "traversal": {1: "per-query stacks", 2: "warp packets"}[ch.traversal],
                   "graph_captured": True, "l2": f"flushed between steps ({L2_FLUSH_BYTES >> 20} MiB write)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "tree_build_s": {f"host_L{plain.levels}": build_plain_s,
                                    f"device_L{plain.levels}": build_plain_dev_s,
                                    f"device_L{ch.levels}": build_chosen_s}, "autotune_s": tune_s},
        "plain": {"value": plain_value, "ms_per_step": t_plain / args.steps, "levels": plain.levels,
                  "threads_per_query": "auto"},
        "chosen_vs_plain": value / plain_value,
        "identical_results_plain_vs_chosen": same,
        "autotune_table": [list(map(lambda x: round(x, 4) if isinstance(x, float) else x, r)) for r in ch.table],
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind, "traffic": traffic, "kernel": kernel_name, "kernel_ms": kern_avg,
                     "algorithmic_bytes_per_launch": alg,
                     "algorithmic_bytes_basis": "1,048,576 x (12 B query + 128 B results) + 12 B per reference "
                                                "point + 8 B per split node",
                     "layout_bytes_per_launch": layout_bytes(n_ref, nq, K_NN, ch.levels),
                     "layout_frac": layout_bytes(n_ref, nq, K_NN, ch.levels) / (kern_avg / 1e3) / 1e9 / peak,
                     "traffic_profile": f"profiles/{prof_tag}.md" if traffic is not None else None,
                     "profiled_shape": shape if traffic is not None else
                     f"no committed profile of this launch shape ({shape})",
                     "binding": "instruction issue (see issue): the search is bound by divergent control flow "
                                "and L2 latency, not by DRAM bandwidth",
                     "issue": issue},
        "cpu_baseline": cpu,
        "exactness_vs_oracle_sample": exact,
        "fp32_dists_vs_fp64_recomputation": fp64,
        "e2e": {"value": world * nq * args.steps / (t_e2e / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": q_host.numel() * 4,
                "d2h_bytes_per_step": d_host.numel() * 4 + i_host.numel() * 4,
                "transfer": "tk_tree_query_host: queries in one H2D copy; results written by the query kernel "
                            "straight into the pinned host buffers",
                "ms_per_step": t_e2e / args.steps},
        # per chosen step (one graph replay): k_bin_count, the three kernels of the
        # cell-count scan (k_scan_tiles, k_scan_single, k_scan_add), k_bin_scatter,
        # the cost-class pass (k_digit_hist, three scan kernels, k_digit_scatter)
        # and the KD query kernel
        "gpu_launches": 11 * args.steps,
        "clocks": clocks,
        "other_workloads": rows,
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(ref_np, q_np, gpu_idx, gpu_d, sample):
    """The oracle's restatement of the reference CPU query, timed on the host
    cores on the first `sample` queries; also checks the GPU's answers for
    that sample against it (distances bitwise, indices up to exact ties)."""
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    L = O.default_levels(len(ref_np))
    lay = O.build_tree(ref_np, L, nthreads=threads)
    qs = q_np[:sample]
    t0 = time.perf_counter()
    od, oi = O.query_tree(lay, qs, K_NN, nthreads=threads)
    dt = time.perf_counter() - t0
    cmp = O.compare_knn(od, oi, gpu_d, gpu_idx)
    cpu = {"value": sample / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"first {sample} of the 1,048,576 queries, full 4,194,304-point tree (levels {L})"}
    exact = {"queries": sample, "index_mismatches_non_tie": cmp.mismatches, "tie_queries": cmp.tie_queries,
             "dist_bit_mismatches": cmp.dist_bit_mismatch}
    return cpu, exact


# ------------------------------------------- the other workloads' rows --
#
# Bounded versions of the other benchmark workloads, run after the headline
# on the same GPU and reported inside its JSON line: each with its own CUDA
# event timing, a roofline against its own bound and exactness against the
# oracle (never against another GPU path).

FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2070e6 / 1e12  # CUDA-core FP32 FMA rate at the maximum SM clock


def measured_peak_bf16():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except (OSError, ValueError, KeyError):
        return 1900.0, "fallback"


def _median(ms):
    return float(statistics.median(ms))


def _cmp_dict(c):
    return {"queries": c.n_queries, "index_mismatches_non_tie": c.mismatches, "tie_queries": c.tie_queries,
            "dist_bit_mismatches": c.dist_bit_mismatch}


def row_plain(dev, steps, warmup, threads):
    """Plain KD query: 100,000 refs and 10,000 queries N(0,1)*1e3, k=5, the
    reference's default depth; one graph-replayed query vs the oracle's
    restatement of the reference CPU query on the same inputs."""
    import torch

    import torch_kdtree_gb300 as tk
    from oracle import oracle as O
    from torch_kdtree_gb300.nn_distance import knn_query_raw
    from torch_kdtree_gb300.synthetic import plain_cloud
    ref_np, q_np = plain_cloud()
    ref, q = torch.from_numpy(ref_np).to(dev), torch.from_numpy(q_np).to(dev)
    k = 5
    tree = tk.build_kd_tree(ref)
    d = torch.empty(len(q), k, device=dev)
    i = torch.empty(len(q), k, dtype=torch.int32, device=dev)
    s = torch.cuda.Stream(dev)
    s.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(s):
        knn_query_raw(tree._tree, q, k, d, i)
    torch.cuda.current_stream(dev).wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        knn_query_raw(tree._tree, q, k, d, i)
    ms = _median(_event_ms(g.replay, max(steps, 20), warmup))
    g.replay()
    torch.cuda.synchronize()
    lay = O.build_tree(ref_np, O.default_levels(len(ref_np)), nthreads=threads)
    t0 = time.perf_counter()
    od, oi = O.query_tree(lay, q_np, k, nthreads=threads)
    cpu_s = time.perf_counter() - t0
    alg = algorithmic_bytes(len(ref_np), len(q_np), k, tree.levels)
    peak, kind = measured_peak_hbm()
    return {"workload": "100,000 refs x 10,000 queries N(0,1)*1e3, d=3, k=5, levels 13 (reference default), "
                        "graph-replayed", "value": len(q_np) / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak, "peak_kind": kind,
                         "unit": "GB/s", "frac": alg / (ms / 1e3) / 1e9 / peak, "algorithmic_bytes_per_launch": alg,
                         "binding": "launch and latency: 10,000 queries are a fraction of one wave"},
            "cpu_baseline": {"value": len(q_np) / cpu_s, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "all 10,000 queries"},
            "exactness_vs_oracle": _cmp_dict(O.compare_knn(od, oi, d.cpu().numpy(), i.cpu().numpy()))}


def row_backward(dev, steps, warmup, flush, threads):
    """Differentiable KNN: 1,048,576 refs and queries N(0,1), k=8, loss =
    0.5 * sum(dists * w): forward query vs the hand-written backward, the
    gradient against the reference's torch-indexed formula and against FP64
    central differences (step 1e-4) on the first 4,096 queries, the forward
    against the oracle on a query sample."""
    import torch

    import torch_kdtree_gb300 as tk
    from oracle import oracle as O
    from torch_kdtree_gb300._lib import QueryOpts
    from torch_kdtree_gb300.autograd import knn_backward
    from torch_kdtree_gb300.nn_distance import knn_query_raw
    from torch_kdtree_gb300.synthetic import differentiable
    ref_np, q_np, w_np = differentiable()
    ref, q, w = (torch.from_numpy(a).to(dev) for a in (ref_np, q_np, w_np))
    k, n = 8, len(ref_np)
    tree = tk.build_kd_tree(ref, levels=16, query_opts=QueryOpts.make(threads_per_query=1))
    d = torch.empty(n, k, device=dev)
    i = torch.empty(n, k, dtype=torch.int32, device=dev)
    fwd = _median(_event_ms(lambda: knn_query_raw(tree._tree, q, k, d, i, tree.query_opts), steps, warmup, flush))
    g = 0.5 * w
    bwd = _median(_event_ms(lambda: knn_backward(q, ref, i, g, True, True), steps, warmup, flush))
    gq, gr = knn_backward(q, ref, i, g, True, True)
    # the reference's gradient: torch autograd through dists re-gathered by index (nn_distance.py:111-112)
    qq, rr = q.clone().requires_grad_(True), ref.clone().requires_grad_(True)
    dd = ((qq[:, None, :] - rr[i.long()]) ** 2).sum(-1)
    tq, tr = torch.autograd.grad((dd * g).sum(), (qq, rr))
    rel = lambda a, b: float((a - b).abs().max() / b.abs().max().clamp_min(1e-30))
    # FP64 central differences (step 1e-4) of the loss with the neighbour
    # lists held fixed (the loss is differentiable wherever no two neighbours
    # swap ranks): every coordinate of the first 4,096 queries, and of 64
    # reference points that are neighbours of them
    m, h = 4096, 1e-4
    q64, r64, g64, il = q.double(), ref.double(), g.double(), i.long()
    fd = torch.empty(m, 3, dtype=torch.float64, device=dev)
    for c in range(3):
        e = torch.zeros(m, 3, dtype=torch.float64, device=dev)
        e[:, c] = h
        lp = (((q64[:m] + e)[:, None] - r64[il[:m]]) ** 2).sum(-1).mul(g64[:m]).sum(1)
        lm = (((q64[:m] - e)[:, None] - r64[il[:m]]) ** 2).sum(-1).mul(g64[:m]).sum(1)
        fd[:, c] = (lp - lm) / (2 * h)
    err_q = ((gq[:m].double() - fd).abs() / fd.abs().clamp_min(1e-3)).max()
    refs_checked = torch.unique(il[:m, 0])[:64]
    err_r = 0.0
    for mm in refs_checked.tolist():
        rows, cols = (il == mm).nonzero(as_tuple=True)
        for c in range(3):
            def part(rv):
                return ((q64[rows] - rv) ** 2).sum(-1).mul(g64[rows, cols]).sum()
            e = torch.zeros(3, dtype=torch.float64, device=dev)
            e[c] = h
            f = float((part(r64[mm] + e) - part(r64[mm] - e)) / (2 * h))
            err_r = max(err_r, abs(float(gr[mm, c]) - f) / max(abs(f), 1e-3))
    fd_rel = max(float(err_q), err_r)
    # forward exactness on a sample
    sample = 65536
    lay = O.build_tree(ref_np, O.default_levels(n), nthreads=threads)
    od, oi = O.query_tree(lay, q_np[:sample], k, nthreads=threads)
    cmp = O.compare_knn(od, oi, d[:sample].cpu().numpy(), i[:sample].cpu().numpy())
    alg = n * k * (4 + 4 + 12) + n * 24 + n * 12
    peak, kind = measured_peak_hbm()
    return {"workload": "1,048,576 refs + 1,048,576 queries N(0,1), d=3, k=8, loss 0.5*sum(dists*w), w U(0,1); "
                        "levels 16, one lane per query", "forward_ms": fwd, "backward_ms": bwd,
            "value": bwd / fwd, "unit": "backward / forward time", "target": "< 1.5",
            "roofline": {"bound": "hbm", "kernel": "backward (all its kernels)", "achieved": alg / (bwd / 1e3) / 1e9,
                         "peak": peak, "peak_kind": kind, "unit": "GB/s", "frac": alg / (bwd / 1e3) / 1e9 / peak,
                         "algorithmic_bytes_per_launch": alg,
                         "algorithmic_bytes_basis": "Q k (4 idx + 4 grad + 12 gather) + Q 24 (q in, dq out) + "
                                                    "N 12 (dref out)"},
            "gradient_vs_torch_indexed": {"grad_q_max_rel": rel(gq, tq), "grad_ref_max_rel": rel(gr, tr)},
            "gradient_vs_fp64_central_differences": {"queries": m, "reference_points": len(refs_checked),
                                                     "step": h, "neighbour_lists": "held fixed",
                                                     "max_rel_err": fd_rel, "tolerance": 1e-3,
                                                     "rel_err_floor": "denominator at least 1e-3"},
            "forward_exactness_vs_oracle": _cmp_dict(cmp)}


def row_batched(dev, steps, warmup, flush, threads):
    """256 ragged clouds (sizes log-uniform in [1e3, 2e5], 8-Gaussian
    mixtures, queries = half the size, k from {1, 4, 16}): one graph-captured
    persistent launch vs one launch per cloud; 16 clouds checked against the
    oracle (the largest, the smallest and spread sizes, every k)."""
    import torch

    from oracle import oracle as O
    from torch_kdtree_gb300.batched import BatchedKDTrees
    from torch_kdtree_gb300.synthetic import ragged_clouds
    clouds = ragged_clouds(n_clouds=256, seed=0)
    refs = [torch.from_numpy(r).to(dev) for r, _, _ in clouds]
    qs = [torch.from_numpy(q).to(dev) for _, q, _ in clouds]
    ks = [k for _, _, k in clouds]
    qc = [len(q) for q in qs]
    q_flat = torch.cat(qs).contiguous()
    total_q = len(q_flat)
    tuned_levels = [int(max(1, min(24, round(np.log2(max(2, len(r)) / 16))))) for r, _, _ in clouds]
    plain = BatchedKDTrees(refs, ks, qc)  # the reference's depth per cloud
    tuned = BatchedKDTrees(refs, ks, qc, levels=tuned_levels)
    ms_plain = sum(_event_ms(lambda: plain.query_each(qs), steps, warmup, flush)) / steps
    replay = tuned.graph(q_flat)
    ms_batch = sum(_event_ms(replay, steps, warmup, flush)) / steps
    plain.query_each(qs)
    replay()
    torch.cuda.synchronize()
    same = bool(torch.equal(plain.out_dists, tuned.out_dists) and torch.equal(plain.out_idx, tuned.out_idx))
    sizes = np.array([len(r) for r, _, _ in clouds])
    by_size = np.argsort(sizes)
    pick = {int(by_size[0]), int(by_size[-1])}
    for kk in (1, 4, 16):
        cand = [c for c in by_size[::-1] if ks[c] == kk]
        pick.update(int(c) for c in cand[:: max(1, len(cand) // 4)][:4])
    for c in by_size[:: max(1, len(by_size) // 16)]:
        if len(pick) >= 16:
            break
        pick.add(int(c))
    checks = []
    d_split, i_split = tuned.split(tuned.out_dists), tuned.split(tuned.out_idx)
    for c in sorted(pick):
        r_np, q_np, kk = clouds[c]
        lay = O.build_tree(r_np, O.default_levels(len(r_np)), nthreads=threads)
        od, oi = O.query_tree(lay, q_np, kk, nthreads=threads)
        checks.append(O.compare_knn(od, oi, d_split[c].cpu().numpy(), i_split[c].cpu().numpy()))
    alg = sum(q * (12 + 8 * k) + 12 * len(r) + 8 * ((1 << L) - 1)
              for (r, _, _), q, k, L in zip(clouds, qc, ks, tuned_levels))
    peak, kind = measured_peak_hbm()
    return {"workload": f"256 clouds, {int(sizes.sum())} refs, {total_q} queries, k in {{1,4,16}}, d=3; tuned "
                        "depth (~16 points per leaf)",
            "value": total_q / (ms_batch / 1e3), "unit": UNIT, "ms_per_step": ms_batch,
            "plain_256_launches": {"value": total_q / (ms_plain / 1e3), "ms_per_step": ms_plain},
            "batched_vs_plain": ms_plain / ms_batch, "identical_results_batched_vs_plain": same,
            "roofline": {"bound": "hbm", "achieved": alg / (ms_batch / 1e3) / 1e9, "peak": peak, "peak_kind": kind,
                         "unit": "GB/s", "frac": alg / (ms_batch / 1e3) / 1e9 / peak,
                         "algorithmic_bytes_per_launch": alg, "kernel": "k_batch_query",
                         "traffic": profiled_traffic("batch_query_256_ragged"),
                         "traffic_profile": "profiles/batch_query_256_ragged.md"
                         if profiled_traffic("batch_query_256_ragged") is not None else None},
            "exactness_vs_oracle": {"clouds": len(pick), "queries": int(sum(c.n_queries for c in checks)),
                                    "index_mismatches_non_tie": int(sum(c.mismatches for c in checks)),
                                    "tie_queries": int(sum(c.tie_queries for c in checks)),
                                    "dist_bit_mismatches": int(sum(c.dist_bit_mismatch for c in checks))}}


def row_brute_tc(dev, steps, warmup, threads):
    """Tensor-core brute force: 262,144 refs, 65,536 queries N(0,1) in d = 8
    and 32 with 5% exact duplicate refs, k=32; FP32 CUDA cores vs TF32 and
    BF16 hi/lo products (over-fetch 2k, exact re-rank); every mode checked
    against the oracle's exhaustive search on the first 1,024 queries."""
    import torch

    from oracle import oracle as O
    from torch_kdtree_gb300.nn_distance import nn_distance_raw
    from torch_kdtree_gb300.synthetic import tensor_core_brute
    k, sample = 32, 1024
    bf16, bkind = measured_peak_bf16()
    peaks = {"exact": (FP32_NOMINAL_TFLOPS, "nominal FP32 CUDA-core rate at the maximum clock"),
             "tf32": (bf16 / 2, f"half the {bkind} dense BF16 rate (TF32 runs at half the BF16 rate)"),
             "bf16_split": (bf16, f"{bkind} dense BF16 rate")}
    out = {}
    for dim in (8, 32):
        ref_np, q_np = tensor_core_brute(d=dim)
        ref, q = torch.from_numpy(ref_np).to(dev), torch.from_numpy(q_np).to(dev)
        od, oi = O.brute(ref_np, q_np[:sample], k, nthreads=threads)
        pairs = len(ref_np) * len(q_np)
        res = {}
        for mode in ("exact", "tf32", "bf16_split"):
            dd = torch.empty(len(q), k, device=dev)
            ii = torch.empty(len(q), k, dtype=torch.int32, device=dev)
            ms = _median(_event_ms(lambda: nn_distance_raw(ref, q, k, dd, ii, mode), steps, warmup))
            tf = 2 * dim * pairs / (ms / 1e3) / 1e12
            pk, pkind = peaks[mode]
            res[mode] = {"ms": ms, "pairs_per_s": pairs / (ms / 1e3),
                         "roofline": {"bound": "tensor" if mode != "exact" else "fp32", "achieved": tf, "peak": pk,
                                      "peak_kind": pkind, "unit": "TFLOP/s", "frac": tf / pk,
                                      "basis": "2d flops per (query, reference) pair; selection and re-rank "
                                               "not counted"},
                         "exactness_vs_oracle": _cmp_dict(O.compare_knn(od, oi, dd[:sample].cpu().numpy(),
                                                                        ii[:sample].cpu().numpy()))}
            if mode != "exact":
                res[mode]["speedup_vs_exact"] = res["exact"]["ms"] / ms
        out[f"d{dim}"] = res
        del ref, q
    best = min(out["d32"]["tf32"]["ms"], out["d32"]["bf16_split"]["ms"])
    return {"workload": "262,144 refs x 65,536 queries N(0,1), 5% duplicate refs, k=32, d in {8, 32}",
            "value": out["d32"]["exact"]["ms"] / best, "unit": "x (tensor-core over FP32 brute force, d=32)",
            "runs": out}


def run_rows(args, dev, flush):
    """The other workloads' rows, each bounded to a few seconds."""
    threads = os.cpu_count() or 1
    steps, warmup = max(3, min(args.steps, 5)), 2
    rows = {}
    for name, fn in (("plain_c1", lambda: row_plain(dev, steps, warmup, threads)),
                     ("backward_c3", lambda: row_backward(dev, steps, warmup, flush, threads)),
                     ("batched_c4", lambda: row_batched(dev, steps, warmup, flush, threads)),
                     ("brute_tc_c5", lambda: row_brute_tc(dev, steps, warmup, threads))):
        t0 = time.perf_counter()
        rows[name] = fn()
        rows[name]["wall_s"] = time.perf_counter() - t0
    return rows

# ------------------------------------------------------ other workloads --

def _event_ms(fn, steps, warmup, flush=None):
    import torch
    for _ in range(warmup):
        if flush is not None:
            flush.zero_()
        fn()
    torch.cuda.synchronize()
    ms = []
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        ms.append(a.elapsed_time(b))
    return ms


def run_batched(args):
    """256 ragged clouds (sizes log-uniform in [1e3, 2e5], 8-Gaussian
    mixtures, queries = half the size, k from {1, 4, 16}): one graph-captured
    persistent launch vs one launch per cloud."""
    import torch

    from torch_kdtree_gb300.batched import BatchedKDTrees
    from torch_kdtree_gb300.synthetic import ragged_clouds
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    clouds = ragged_clouds(n_clouds=256, seed=0)
    refs = [torch.from_numpy(r).to(dev) for r, _, _ in clouds]
    qs = [torch.from_numpy(q).to(dev) for _, q, _ in clouds]
    ks = [k for _, _, k in clouds]
    qc = [q.shape[0] for q in qs]
    q_flat = torch.cat(qs).contiguous()
    total_q = q_flat.shape[0]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    leaf = args.leaf_size
    tuned_levels = [int(max(1, min(24, round(np.log2(max(2, len(r)) / leaf))))) for r, _, _ in clouds]
    if args.profile:  # the tuned batch once (trees built on the host: few launches before the batched kernel)
        b = BatchedKDTrees([torch.from_numpy(r) for r, _, _ in clouds], ks, qc, levels=tuned_levels, device=dev)
        b.graph(q_flat)()
        torch.cuda.synchronize()
        return
    t0 = time.perf_counter()
    plain = BatchedKDTrees(refs, ks, qc)  # reference heuristic depth per cloud
    tuned = BatchedKDTrees(refs, ks, qc, levels=tuned_levels)
    build_s = time.perf_counter() - t0
    ms_plain = _event_ms(lambda: plain.query_each(qs), args.steps, args.warmup, flush)
    ms_each_tuned = _event_ms(lambda: tuned.query_each(qs), args.steps, args.warmup, flush)
    replay = tuned.graph(q_flat)
    ms_batch = _event_ms(replay, args.steps, args.warmup, flush)
    plain.query_each(qs)
    replay()
    torch.cuda.synchronize()
    same = bool(torch.equal(plain.out_dists, tuned.out_dists) and torch.equal(plain.out_idx, tuned.out_idx))
    t_b = sum(ms_batch) / 1e3
    value = total_q * args.steps / t_b
    line = {
        "metric": "KNN queries/s, 256 ragged clouds (d=3, k in {1,4,16}), one graph-captured launch vs 256 plain launches",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_b / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded numpy mixtures)",
        "config": {"workload": f"256 clouds, {sum(len(r) for r, _, _ in clouds)} ref points, {total_q} queries",
                   "tuned_leaf_size": leaf, "l2": "flushed between steps", "tree_build_s": build_s},
        "plain_256_launches": {"value": total_q * args.steps / (sum(ms_plain) / 1e3),
                               "ms_per_step": sum(ms_plain) / args.steps},
        "tuned_trees_256_launches": {"value": total_q * args.steps / (sum(ms_each_tuned) / 1e3),
                                     "ms_per_step": sum(ms_each_tuned) / args.steps},
        "batched_vs_plain": (sum(ms_plain) / sum(ms_batch)),
        "identical_results": same,
    }
    print(json.dumps(line), flush=True)


def run_backward(args):
    """Differentiable KNN: 1,048,576 refs and queries N(0,1), k=8, loss =
    0.5 * sum(dists * w); forward query vs the hand-written backward."""
    import torch

    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300._lib import QueryOpts
    from torch_kdtree_gb300.autograd import knn_backward
    from torch_kdtree_gb300.nn_distance import knn_query_raw
    from torch_kdtree_gb300.synthetic import differentiable
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ref_np, q_np, w_np = differentiable()
    ref = torch.from_numpy(ref_np).to(dev)
    q = torch.from_numpy(q_np).to(dev)
    w = torch.from_numpy(w_np).to(dev)
    k = 8
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    res = {}
    for name, levels, tpq in (("plain", None, 0), ("chosen", args.levels or 16, args.tpq or 1)):
        tree = tk.build_kd_tree(ref, levels=levels, query_opts=QueryOpts.make(threads_per_query=tpq))
        d = torch.empty(len(q), k, device=dev)
        i = torch.empty(len(q), k, dtype=torch.int32, device=dev)
        fwd = _event_ms(lambda: knn_query_raw(tree._tree, q, k, d, i, tree.query_opts), args.steps, args.warmup,
                        flush)
        g = 0.5 * w
        bwd = _event_ms(lambda: knn_backward(q, ref, i, g, True, True), args.steps, args.warmup, flush)
        res[name] = {"levels": tree.levels, "forward_ms": sum(fwd) / len(fwd), "backward_ms": sum(bwd) / len(bwd)}
        res[name]["backward_over_forward"] = res[name]["backward_ms"] / res[name]["forward_ms"]
    line = {
        "metric": "backward time / forward time, differentiable KNN (1M refs, 1M queries, d=3, k=8)",
        "value": res["chosen"]["backward_over_forward"], "unit": "ratio", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": res["chosen"]["backward_ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy)",
        "config": {"workload": "1,048,576 refs + 1,048,576 queries N(0,1), k=8, w U(0,1)",
                   "l2": "flushed between steps"},
        "runs": res,
    }
    print(json.dumps(line), flush=True)


def run_brute(args):
    """Brute-force nn_distance on the 65,536 x 65,536 subset of the large
    workload, k = 1, float32 CUDA cores, the reference's arithmetic."""
    import torch

    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300.nn_distance import nn_distance_raw
    from torch_kdtree_gb300.synthetic import cube_and_sphere
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ref_np, q_np = cube_and_sphere()
    ref = torch.from_numpy(ref_np[:65536]).to(dev)
    q = torch.from_numpy(q_np[:65536]).to(dev)
    d = torch.empty(65536, 1, device=dev)
    i = torch.empty(65536, 1, dtype=torch.int32, device=dev)
    ms = _event_ms(lambda: nn_distance_raw(ref, q, 1, d, i, "exact"), args.steps, args.warmup)
    kd, ki = tk.build_kd_tree(ref).query(q, nr_nns_searches=1)
    t = sum(ms) / len(ms) / 1e3
    pairs = 65536 * 65536
    line = {
        "metric": "brute-force KNN pairs/s (65,536 x 65,536, d=3, k=1, float32 exact)",
        "value": pairs / t, "unit": "pairs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (first 65,536 refs and queries of the large workload)",
        "config": {"workload": "nn_distance 65,536 x 65,536, k=1"},
        "queries_per_s": 65536 / t, "gflops_2d_per_pair": 6 * pairs / t / 1e9,
        "identical_to_kdtree": bool(torch.equal(kd, d) and torch.equal(ki, i)),
    }
    print(json.dumps(line), flush=True)



def run_readme(args):
    """The reference's own benchmark setting (its README plot): references and
    queries N(0,1) * 1e3 in 3-D, default tree depth, query() called on a host
    tensor and followed by a synchronize, timed on the wall clock (as its
    benchmark script does), here at its largest size, 1e6 x 1e6, for k = 1, 10
    and 100.  Also reported: the same query with device-resident inputs (CUDA
    events) and the published RTX 3090 readings of that plot."""
    import numpy as np
    import torch

    import torch_kdtree_gb300 as tk
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(0)
    n = nq = 1_000_000
    ref = torch.from_numpy((rng.standard_normal((n, 3)) * 1e3).astype(np.float32)).to(dev)
    q_host = torch.from_numpy((rng.standard_normal((nq, 3)) * 1e3).astype(np.float32))
    q_dev = q_host.to(dev)
    tree = tk.build_kd_tree(ref)
    published = {1: "1e7-3e7", 10: "~1e7", 100: "2e6-4e6"}  # q/s, visual readings of the plot
    runs = {}
    for k in (1, 10, 100):
        def call():
            tree.query(q_host, nr_nns_searches=k)
            torch.cuda.synchronize()
        for _ in range(max(args.warmup, 1)):
            call()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            call()
        wall = (time.perf_counter() - t0) / args.steps
        ms = _event_ms(lambda: tree.query(q_dev, nr_nns_searches=k), args.steps, args.warmup)
        runs[f"k{k}"] = {"queries_per_s_host_input_wall": nq / wall, "ms_host_input_wall": 1e3 * wall,
                         "queries_per_s_device_resident": nq / (sum(ms) / len(ms) / 1e3),
                         "reference_rtx3090_published_queries_per_s": published[k]}
    line = {
        "metric": "KNN queries/s, reference benchmark setting (1e6 refs x 1e6 queries N(0,1)*1e3, d=3, default depth)",
        "value": runs["k10"]["queries_per_s_host_input_wall"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": runs["k10"]["ms_host_input_wall"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy)",
        "config": {"workload": "torch_kdtree benchmark/benchmark.py setting at 1e6 x 1e6; value = k=10",
                   "levels": tree.levels, "timing": "wall clock around query(host tensor) + synchronize"},
        "runs": runs,
    }
    print(json.dumps(line), flush=True)


def run_plain(args):
    """Plain KD-tree KNN: 100,000 refs and 10,000 queries N(0,1)*1e3, k=5, the
    reference's default depth; GPU query (graph-replayed, inputs resident) vs
    the reference CPU query (oracle restatement) on the same inputs, checked
    for exactness."""
    import torch

    import torch_kdtree_gb300 as tk
    from torch_kdtree_gb300.nn_distance import knn_query_raw
    from torch_kdtree_gb300.synthetic import plain_cloud
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ref_np, q_np = plain_cloud()
    ref = torch.from_numpy(ref_np).to(dev)
    q = torch.from_numpy(q_np).to(dev)
    k = 5
    tree = tk.build_kd_tree(ref)
    d = torch.empty(len(q), k, device=dev)
    i = torch.empty(len(q), k, dtype=torch.int32, device=dev)
    s = torch.cuda.Stream(dev)
    s.wait_stream(torch.cuda.current_stream(dev))
    with torch.cuda.stream(s):
        knn_query_raw(tree._tree, q, k, d, i)
    torch.cuda.current_stream(dev).wait_stream(s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        knn_query_raw(tree._tree, q, k, d, i)
    ms = _event_ms(g.replay, max(args.steps, 20), args.warmup)
    t = sum(ms) / len(ms) / 1e3
    g.replay()
    torch.cuda.synchronize()
    from oracle import oracle as O
    O.build()
    threads = os.cpu_count() or 1
    lay = O.build_tree(ref_np, O.default_levels(len(ref_np)), nthreads=threads)
    t0 = time.perf_counter()
    od, oi = O.query_tree(lay, q_np, k, nthreads=threads)
    cpu_t = time.perf_counter() - t0
    cmp = O.compare_knn(od, oi, d.cpu().numpy(), i.cpu().numpy())
    line = {
        "metric": "KNN queries/s, plain KD-tree (100,000 refs, 10,000 queries N(0,1)*1e3, d=3, k=5)",
        "value": len(q) / t, "unit": UNIT, "n_gpus": 1, "steps": len(ms), "warmup": args.warmup,
        "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded numpy)", "config": {"workload": "plain KD query, levels 13", "graph_captured": True},
        "cpu_baseline": {"value": len(q) / cpu_t, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": "all 10,000 queries"},
        "exactness_vs_reference_cpu": {"index_mismatches_non_tie": cmp.mismatches, "tie_queries": cmp.tie_queries,
                                       "dist_bit_mismatches": cmp.dist_bit_mismatch},
    }
    print(json.dumps(line), flush=True)


def run_wide(args):
    """KD trees of 4, 6 and 8 dimensions (the reference's README recipe for more
    dims): 1,048,576 refs and 262,144 queries N(0,1), k=16, float32; tuned tree
    depth and lanes.  Beside it: the exhaustive exact search on the same
    queries, and the reference's CPU query (oracle restatement, all host
    threads) on the first 16,384 queries, checked for exactness."""
    import numpy as np
    import torch

    import torch_kdtree_gb300 as tk
    from oracle import oracle as O
    from torch_kdtree_gb300.autotune import autotune
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    n, nq, k, sample = 1 << 20, 1 << 18, 16, 16384
    if args.profile:  # one d=8 query of 65,536 queries, tuned shape (levels 12, 32 lanes, split planes only)
        from torch_kdtree_gb300._lib import QueryOpts
        rng = np.random.default_rng(48)
        ref = torch.from_numpy(rng.standard_normal((n, 8)).astype(np.float32)).to(dev)
        q = torch.from_numpy(rng.standard_normal((65536, 8)).astype(np.float32)).to(dev)
        tree = tk.build_kd_tree(ref, levels=12, query_opts=QueryOpts.make(threads_per_query=32, prune_boxes=0))
        tree.query(q, nr_nns_searches=k)
        torch.cuda.synchronize()
        return
    O.build()
    threads = os.cpu_count() or 1
    runs = {}
    for d in (4, 6, 8):
        rng = np.random.default_rng(40 + d)
        ref_np = rng.standard_normal((n, d)).astype(np.float32)
        q_np = rng.standard_normal((nq, d)).astype(np.float32)
        ref, q = torch.from_numpy(ref_np).to(dev), torch.from_numpy(q_np).to(dev)
        ch = autotune(ref, q, k, use_cache=False, max_queries=65536)
        tree = tk.build_kd_tree(ref, levels=ch.levels, query_opts=ch.opts())
        ms = _event_ms(lambda: tree.query(q, nr_nns_searches=k), args.steps, args.warmup)
        kd_t = sum(ms) / len(ms) / 1e3
        bq = q[:65536]
        bms = _event_ms(lambda: tk.nn_distance(ref, bq, k), max(1, args.steps // 2), 1)
        brute_qps = len(bq) / (sum(bms) / len(bms) / 1e3)
        gd, gi = tree.query(q[:sample], nr_nns_searches=k)
        lay = O.build_tree(ref_np, O.default_levels(n), nthreads=threads)
        t0 = time.perf_counter()
        od, oi = O.query_tree(lay, q_np[:sample], k, nthreads=threads)
        cpu_t = time.perf_counter() - t0
        cmp = O.compare_knn(od, oi, gd.cpu().numpy(), gi.cpu().numpy())
        runs[f"d{d}"] = {"queries_per_s": nq / kd_t, "ms": 1e3 * kd_t, "levels": ch.levels,
                         "threads_per_query": ch.threads_per_query, "prune_boxes": ch.prune_boxes,
                         "brute_exact_queries_per_s": brute_qps,
                         "cpu_reference_queries_per_s": sample / cpu_t,
                         "cpu_reference_levels": O.default_levels(n),
                         "exact_vs_cpu": {"index_mismatches_non_tie": cmp.mismatches,
                                          "tie_queries": cmp.tie_queries,
                                          "dist_bit_mismatches": cmp.dist_bit_mismatch}}
        del tree, ref, q
    line = {
        "metric": "KNN queries/s, KD trees of 4-8 dims (1,048,576 refs x 262,144 queries N(0,1), k=16); value = d=6",
        "value": runs["d6"]["queries_per_s"], "unit": UNIT, "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": runs["d6"]["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy)",
        "config": {"workload": "KD query, d in {4, 6, 8}, tuned depth and lanes, inputs resident"},
        "cpu_baseline": {"value": runs["d6"]["cpu_reference_queries_per_s"], "unit": UNIT, "cores": threads,
                         "kind": "port", "sample": f"first {sample} queries, reference default depth"},
        "runs": runs,
    }
    print(json.dumps(line), flush=True)


def run_cpu_tree(args):
    """CPU trees (build_kd_tree(..., device="cpu"), the reference's KDTreeCPU
    path): the library's threaded host search against the reference's CPU
    search (oracle restatement, same threads) on 131,072 queries of the large
    single-cloud workload (4,194,304 refs, k=16), at the reference's default
    depth and at depth 18; exactness against the oracle's answers."""
    import torch

    import torch_kdtree_gb300 as tk
    from oracle import oracle as O
    from torch_kdtree_gb300.synthetic import cube_and_sphere
    O.build()
    ref_np, q_all = cube_and_sphere()[:2]
    nq, k = 131072, 16
    q_np = np.ascontiguousarray(q_all[:nq])
    threads = os.cpu_count() or 1
    qt = torch.from_numpy(q_np)
    runs = {}
    for levels in (O.default_levels(len(ref_np)), 18):
        tree = tk.build_kd_tree(torch.from_numpy(ref_np), device="cpu", levels=levels)
        lay = O.build_tree(ref_np, levels, nthreads=threads)
        ours = ora = 1e30
        tree.query(qt[:4096], nr_nns_searches=k)  # warm-up: host threads started, pages touched
        O.query_tree(lay, q_np[:4096], k, nthreads=threads)
        for _ in range(3):
            t0 = time.perf_counter()
            d, i = tree.query(qt, nr_nns_searches=k)
            ours = min(ours, time.perf_counter() - t0)
            t0 = time.perf_counter()
            od, oi = O.query_tree(lay, q_np, k, nthreads=threads)
            ora = min(ora, time.perf_counter() - t0)
        cmp = O.compare_knn(od, oi, d.numpy(), i.numpy())
        runs[f"levels{levels}"] = {"queries_per_s": nq / ours, "reference_cpu_queries_per_s": nq / ora,
                                   "speedup": ora / ours,
                                   "exact_vs_reference_cpu": {"index_mismatches_non_tie": cmp.mismatches,
                                                              "tie_queries": cmp.tie_queries,
                                                              "dist_bit_mismatches": cmp.dist_bit_mismatch}}
    key = f"levels{O.default_levels(len(ref_np))}"
    line = {
        "metric": "KNN queries/s of CPU trees (host search), 4,194,304 refs, k=16; value = the reference's default depth",
        "value": runs[key]["queries_per_s"], "unit": UNIT, "n_gpus": 0, "steps": 3,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded numpy)",
        "config": {"workload": f"CPU tree query, {nq} of the large single-cloud queries, best of 3 calls",
                   "host_threads": threads},
        "runs": runs,
    }
    print(json.dumps(line), flush=True)


def run_brute_tc(args):
    """Tensor-core brute force vs the FP32 CUDA-core brute force: 262,144 refs,
    65,536 queries, N(0,1) in d = 8 and 32 with 5% exact duplicate refs, k=32.
    The tensor-core modes over-fetch 2k candidates, re-rank them exactly and
    recompute uncertified queries exactly; all modes must agree bit for bit."""
    import torch

    from torch_kdtree_gb300.nn_distance import nn_distance_raw
    from torch_kdtree_gb300.synthetic import tensor_core_brute
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    k = 32
    out = {}
    if args.profile:
        # one tensor-core and one exact call on a reduced query set (for ncu captures)
        ref_np, q_np = tensor_core_brute(d=32, n_query=16384)
        ref = torch.from_numpy(ref_np).to(dev)
        q = torch.from_numpy(q_np).to(dev)
        dd = torch.empty(len(q), k, device=dev)
        ii = torch.empty(len(q), k, dtype=torch.int32, device=dev)
        nn_distance_raw(ref, q, k, dd, ii, "tf32")
        nn_distance_raw(ref, q, k, dd, ii, "exact")
        torch.cuda.synchronize()
        return
    for d in (8, 32):
        ref_np, q_np = tensor_core_brute(d=d)
        ref = torch.from_numpy(ref_np).to(dev)
        q = torch.from_numpy(q_np).to(dev)
        res = {}
        base = None
        for mode in ("exact", "tf32", "bf16_split"):
            dd = torch.empty(len(q), k, device=dev)
            ii = torch.empty(len(q), k, dtype=torch.int32, device=dev)
            ms = _event_ms(lambda: nn_distance_raw(ref, q, k, dd, ii, mode), args.steps, args.warmup)
            t = sum(ms) / len(ms) / 1e3
            pairs = len(ref) * len(q)
            r = {"ms": 1e3 * t, "pairs_per_s": pairs / t, "tflops_2d": 2 * d * pairs / t / 1e12}
            if base is None:
                base = (dd.clone(), ii.clone())
            else:
                r["rows_with_index_mismatch_vs_exact"] = int((ii != base[1]).any(1).sum().item())
                r["dist_bit_mismatch_vs_exact"] = int((dd.view(torch.int32) != base[0].view(torch.int32)).sum().item())
                r["speedup_vs_exact"] = res["exact"]["ms"] / r["ms"]
            res[mode] = r
        out[f"d{d}"] = res
    best = min(out["d32"]["tf32"]["ms"], out["d32"]["bf16_split"]["ms"])
    line = {
        "metric": "tensor-core brute-force speed-up over FP32 brute force at d=32 (262,144 x 65,536, k=32, exact)",
        "value": out["d32"]["exact"]["ms"] / best, "unit": "x", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": best, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 inputs (tf32 / bf16 hi-lo products, fp32 re-rank)",
        "data": "synthetic (seeded numpy N(0,1), 5% duplicate refs)",
        "config": {"workload": "262,144 refs x 65,536 queries, d in {8, 32}, k=32, over-fetch 2k"},
        "runs": out,
    }
    print(json.dumps(line), flush=True)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--ref-sample", type=int, default=131072)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-rows", action="store_true", help="skip the other workloads' rows after the headline")
    p.add_argument("--levels", type=int, default=0, help="chosen tree depth (skips the autotuner with --tpq)")
    p.add_argument("--tpq", type=int, default=0, help="chosen lanes per query (skips the autotuner with --levels)")
    p.add_argument("--boxes", type=int, default=1, help="chosen: prune with node bounding boxes (with --levels/--tpq)")
    p.add_argument("--traversal", type=int, default=1, choices=[1, 2],
                   help="chosen: 1 = per-query stacks, 2 = warp packets (with --levels/--tpq)")
    p.add_argument("--profile", action="store_true", help="run one chosen and one plain query only (for ncu)")
    p.add_argument("--workload", default="kd",
                   choices=["kd", "plain", "readme", "batched", "backward", "brute", "brute_tc", "wide", "cpu_tree"],
                   help="kd (default): the headline large single-cloud query; the others measure the "
                        "batched, backward and brute-force paths")
    p.add_argument("--leaf-size", type=int, default=16, help="target points per leaf of tuned batch trees")
    args = p.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.workload != "kd":
        if rank == 0:
            {"plain": run_plain, "readme": run_readme, "batched": run_batched, "backward": run_backward,
             "brute": run_brute,
             "brute_tc": run_brute_tc, "wide": run_wide, "cpu_tree": run_cpu_tree}[args.workload](args)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    run_ours(args, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
