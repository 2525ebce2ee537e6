"""Generate the golden fixtures from the reference's own CPU KD-tree.

Runs where the reference checkout exists: it builds ``oracle/_ref/libtkref.so``
from the reference's sources (``make -C oracle ref``), then, for a set of
seeded inputs, records the reference's layout (structured points, shuffled
indices, split planes, leaves) and its query output (squared distances and
original indices).  Inputs are regenerated from their seed by
``golden_inputs()`` and guarded by a checksum, so the fixtures stay small.

    python tests/golden/make_golden.py [--force]

The fixtures pin the oracle (tests/test_oracle.py) and serve as a second,
reference-produced check of the GPU path (tests/test_kdtree_gpu.py).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))

# (name, dtype, d, n, nq, k, levels or None, kind, full_output)
CASES = [
    *[(f"grid_{dt}_d{d}_n{n}_q{nq}_k{k}", dt, d, n, nq, k, None, "normal1e3", True)
      for dt in ("f32", "f64") for d in (1, 2, 3)
      for (n, nq, k) in ((5, 5, 1), (30, 20, 5), (1000, 200, 10), (10000, 300, 20))],
    *[(f"levels_f32_d3_n1000_L{L}", "f32", 3, 1000, 100, 7, L, "normal1e3", True) for L in (1, 2, 5, 9)],
    ("ties_f32_d3_grid", "f32", 3, 2000, 300, 8, None, "intgrid", True),
    ("ties_f64_d2_grid", "f64", 2, 1500, 200, 6, None, "intgrid", True),
    ("dup5pct_f32_d3", "f32", 3, 5000, 400, 16, None, "dup5", True),
    # more dimensions, as the reference's README recipe compiles them
    *[(f"wide_{dt}_d{d}_n{n}_q{nq}_k{k}", dt, d, n, nq, k, None, "normal1e3", True)
      for (dt, d, n, nq, k) in (("f32", 4, 1000, 200, 10), ("f32", 5, 10000, 300, 20), ("f32", 8, 10000, 300, 16),
                                ("f64", 6, 1000, 200, 10), ("f64", 8, 5000, 200, 33), ("f32", 7, 30, 20, 5))],
    ("wide_ties_f32_d4_grid", "f32", 4, 2000, 300, 8, None, "intgrid", True),
    # the plain workload: N(0,1)*1e3, 100,000 refs, 10,000 queries, k=5, levels 13
    ("config1_f32_d3_n100000_q10000_k5", "f32", 3, 100000, 10000, 5, None, "normal1e3", False),
]

SUBSET = 1000  # rows of the query output stored in full for large cases


def golden_inputs(name: str, dtype: str, d: int, n: int, nq: int, kind: str):
    """Seeded inputs of a case (seed derived from the case name)."""
    seed = int.from_bytes(hashlib.sha256(name.encode()).digest()[:4], "little")
    rng = np.random.default_rng(seed)
    dt = np.float32 if dtype == "f32" else np.float64
    if kind == "normal1e3":
        ref = rng.standard_normal((n, d)) * 1e3
        q = rng.standard_normal((nq, d)) * 1e3
    elif kind == "intgrid":
        ref = rng.integers(-6, 7, size=(n, d)).astype(np.float64)
        q = rng.integers(-7, 8, size=(nq, d)).astype(np.float64) + 0.5 * rng.integers(0, 2, size=(nq, d))
    elif kind == "dup5":
        ref = rng.standard_normal((n, d))
        m = n // 20
        dst = rng.permutation(n)[:m]
        src = rng.integers(0, n, size=m)
        ref[dst] = ref[src]
        q = rng.standard_normal((nq, d))
    else:
        raise ValueError(kind)
    return np.ascontiguousarray(ref.astype(dt)), np.ascontiguousarray(q.astype(dt))


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main() -> None:
    sys.path.insert(0, ROOT)
    from oracle import oracle as O

    O.build(ref=True)
    force = "--force" in sys.argv
    for (name, dtype, d, n, nq, k, levels, kind, full) in CASES:
        if not force and os.path.exists(os.path.join(HERE, name + ".npz")):
            continue  # fixtures are deterministic; regenerate all with --force
        ref, q = golden_inputs(name, dtype, d, n, nq, kind)
        T = O.RefTree(ref, levels)
        lay = T.layout()
        dists, idx = T.query(q, k)
        out = dict(name=name, dtype=dtype, d=d, n=n, nq=nq, k=k, kind=kind, levels=T.levels,
                   input_sha=digest(ref, q), output_sha=digest(dists, idx),
                   layout_sha=digest(lay.structured, lay.perm, lay.medians, lay.axes, lay.leaf_off,
                                     lay.leaf_cnt))
        rows = nq if full else SUBSET
        out["dists"] = dists[:rows]
        out["idx"] = idx[:rows]
        if full and n <= 10000:
            out.update(structured=lay.structured, perm=lay.perm, medians=lay.medians, axes=lay.axes,
                       leaf_off=lay.leaf_off, leaf_cnt=lay.leaf_cnt)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "levels", T.levels, "rows", rows)


if __name__ == "__main__":
    main()
