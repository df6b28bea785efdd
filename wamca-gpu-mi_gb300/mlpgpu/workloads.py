"""Seeded synthetic workloads of the benchmark configurations (pure numpy).

The reference measures on TSPLIB/TRP instances; these generators stand in for
them with the shapes and distributions the configurations name: integer
coordinates in [0, box]^2 (uniform, or 8 Gaussian clusters with sigma 50 and
centres uniform in the box, rounded and clipped), a depot at node 0 and start
tours made of depot 0, a seeded random permutation of 1..n-1 and depot 0.
"""
from __future__ import annotations

import numpy as np


def uniform_instance(n: int, seed: int, box: int = 1000):
    r = np.random.default_rng(seed)
    return r.integers(0, box + 1, n).astype(np.int32), r.integers(0, box + 1, n).astype(np.int32)


def clustered_instance(n: int, seed: int, clusters: int = 8, sigma: float = 50.0, box: int = 1000):
    r = np.random.default_rng(seed)
    centres = r.uniform(0, box, size=(clusters, 2))
    lab = r.integers(0, clusters, n)
    pts = centres[lab] + r.normal(0.0, sigma, size=(n, 2))
    pts = np.clip(np.rint(pts), 0, box).astype(np.int32)
    return pts[:, 0].copy(), pts[:, 1].copy()


def random_perm_tour(n: int, seed: int) -> np.ndarray:
    r = np.random.default_rng(seed + 1_000_003)
    return np.concatenate([[0], 1 + r.permutation(n - 1), [0]]).astype(np.int32)


def log_uniform_sizes(count: int, lo: int, hi: int, seed: int) -> np.ndarray:
    """count sizes n = round(exp(U[ln lo, ln hi]))."""
    r = np.random.default_rng(seed)
    return np.rint(np.exp(r.uniform(np.log(lo), np.log(hi), count))).astype(np.int32)
