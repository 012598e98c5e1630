"""Seeded inputs of the golden fixtures (shared by make_golden.py and the tests)."""
from __future__ import annotations

import numpy as np

from quantization_graph_gb300 import synthetic


def kernel_inputs(dim: int, n: int, nq: int, seed: int):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, dim)).astype(np.float32) * rng.uniform(0.3, 2.0, dim).astype(np.float32)
    Q = rng.standard_normal((nq, dim)).astype(np.float32) * rng.uniform(0.3, 2.0, dim).astype(np.float32)
    return X, Q


def c1_data(n=2000, nq=50):
    """20k x 128 GMM workload, scaled down: 64 components, centres N(0,1), sigma 0.3."""
    X, cent = synthetic.gmm(n, 128, components=64, sigma=0.3, seed=11)
    Q, _ = synthetic.gmm(nq, 128, sigma=0.3, seed=12, centres=cent)
    return X, Q


def c2_data(n=1500, nq=24):
    """|x|, x ~ N(0, Q Lambda Q^T), lambda_i ~ i^-1.2, 960-d (scaled down)."""
    X = synthetic.anisotropic(n, 960, alpha=1.2, seed=21, absolute=True)
    Q = synthetic.anisotropic(nq, 960, alpha=1.2, seed=22, absolute=True)
    return X, Q


def c3_data(n=1000, nq=16):
    """unit-norm anisotropic, lambda_i ~ i^-0.8, 1536-d (scaled down)."""
    X = synthetic.anisotropic(n, 1536, alpha=0.8, seed=31, normalize=True)
    Q = synthetic.anisotropic(nq, 1536, alpha=0.8, seed=32, normalize=True)
    return X, Q


SEARCH_CASES = {"search_c1": c1_data, "search_c2": c2_data, "search_c3": c3_data}
