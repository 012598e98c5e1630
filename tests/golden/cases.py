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


# rabitq_build_vamana_graph arguments of the graphs stored in the search fixtures (alpha 1.2,
# beam 1) and of the extra build variants (build_variants.npz) over the same records.
SEARCH_GRAPH_ARGS = {
    "search_c1": dict(r=32, l_build=100, alpha=1.2, beam=1, batch=256, refine=1, cap=256, stop_hops=2),
    "search_c2": dict(r=32, l_build=64, alpha=1.2, beam=1, batch=256, refine=1, cap=256, stop_hops=2),
    "search_c3": dict(r=32, l_build=64, alpha=1.2, beam=1, batch=256, refine=1, cap=256, stop_hops=2),
}
BUILD_VARIANTS = {
    "beam2_alpha13_cap48": dict(src="search_c1", r=32, l_build=64, alpha=1.3, beam=2, batch=300, refine=0,
                                cap=48, stop_hops=0),
    "alpha1_r16_refine2": dict(src="search_c1", r=16, l_build=40, alpha=1.0, beam=1, batch=1000, refine=2,
                               cap=0, stop_hops=3),
    "alpha2_batch1": dict(src="search_c1", r=8, l_build=24, alpha=2.0, beam=3, batch=1, refine=1, cap=16,
                          stop_hops=1),
    "d960_r24": dict(src="search_c2", r=24, l_build=48, alpha=1.2, beam=1, batch=4096, refine=1, cap=32,
                     stop_hops=2),
}


def build_edge_data():
    """Duplicates, near-duplicates (1e-7 apart) and zero vectors among 128-d Gaussians: equal
    codes, zero and invalid-record distances, ties broken by id."""
    rng = np.random.default_rng(5)
    base = rng.standard_normal((300, 128)).astype(np.float32)
    X = np.concatenate([base, base[:150], base[:75] + np.float32(1e-7), np.zeros((10, 128), np.float32)])
    rng.shuffle(X)
    return X


BUILD_EDGE_ARGS = {
    "edge_r16": dict(r=16, l_build=32, alpha=1.2, beam=1, batch=64, refine=1, cap=24, stop_hops=2),
    "edge_r8_beam2": dict(r=8, l_build=16, alpha=1.0, beam=2, batch=1000, refine=0, cap=0, stop_hops=0),
    "edge_n3": dict(n=3, r=4, l_build=8, alpha=1.2, beam=1, batch=4, refine=1, cap=0, stop_hops=0),
}
