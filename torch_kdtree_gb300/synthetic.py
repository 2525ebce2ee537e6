"""Seeded synthetic inputs with the shapes and distributions of the
benchmark configurations (no public dataset is involved).

All generators use numpy's PCG64 ``default_rng(seed)`` and return float32
numpy arrays, drawing the reference cloud first and the queries second."""
from __future__ import annotations

import numpy as np


def plain_cloud(n_ref=100_000, n_query=10_000, d=3, scale=1e3, seed=0, dtype=np.float32):
    """Plain KD-tree KNN: every coordinate i.i.d. N(0,1) * scale."""
    rng = np.random.default_rng(seed)
    ref = (rng.standard_normal((n_ref, d)) * scale).astype(dtype)
    q = (rng.standard_normal((n_query, d)) * scale).astype(dtype)
    return ref, q


def cube_and_sphere(n_ref=4_194_304, n_query=1_048_576, seed=0, sigma=0.01):
    """Large single cloud: half uniform in [0,1]^3, half on the unit sphere
    centred at (0.5,0.5,0.5) with N(0, sigma) radial noise; queries uniform
    in [-0.1, 1.1]^3."""
    rng = np.random.default_rng(seed)
    h = n_ref // 2
    cube = rng.random((h, 3))
    u = rng.standard_normal((n_ref - h, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = 1.0 + rng.normal(0.0, sigma, size=(n_ref - h, 1))
    sphere = 0.5 + r * u
    ref = np.concatenate([cube, sphere]).astype(np.float32)
    q = (rng.random((n_query, 3)) * 1.2 - 0.1).astype(np.float32)
    return ref, q


def differentiable(n_ref=1_048_576, n_query=1_048_576, k=8, seed=0):
    """Differentiable KNN: ref and queries N(0,1) in 3-D, weights w U(0,1) [Q, k]."""
    rng = np.random.default_rng(seed)
    ref = rng.standard_normal((n_ref, 3)).astype(np.float32)
    q = rng.standard_normal((n_query, 3)).astype(np.float32)
    w = rng.random((n_query, k)).astype(np.float32)
    return ref, q, w


def ragged_clouds(n_clouds=256, lo=1_000, hi=200_000, seed=0):
    """Batched ragged clouds: sizes log-uniform in [lo, hi]; each cloud a
    mixture of 8 isotropic Gaussians (means U(-10,10)^3, sigma U(0.1,2),
    equal weights); queries = floor(0.5 * size) from the same mixture; k per
    cloud from {1, 4, 16}."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_clouds):
        size = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        means = rng.uniform(-10, 10, size=(8, 3))
        sig = rng.uniform(0.1, 2.0, size=8)

        def draw(m):
            comp = rng.integers(0, 8, size=m)
            return (means[comp] + rng.standard_normal((m, 3)) * sig[comp, None]).astype(np.float32)

        ref = draw(size)
        q = draw(size // 2)
        k = int(rng.choice([1, 4, 16]))
        out.append((ref, q, k))
    return out


def tensor_core_brute(n_ref=262_144, n_query=65_536, d=32, dup_frac=0.05, seed=0):
    """Brute-force workload: N(0,1) in d dims, then dup_frac of the reference
    rows (seeded permutation) overwritten by copies of other rows."""
    rng = np.random.default_rng(seed)
    ref = rng.standard_normal((n_ref, d)).astype(np.float32)
    q = rng.standard_normal((n_query, d)).astype(np.float32)
    m = int(round(dup_frac * n_ref))
    perm = rng.permutation(n_ref)
    dst, src = perm[:m], perm[m:2 * m]
    ref[dst] = ref[src]
    return ref, q
