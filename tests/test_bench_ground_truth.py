"""bench.ground_truth: the exact top-k under FP64 distances, certified per query by the FP32
error bound of the shortlist scores, with a full FP64 scan for the queries the bound cannot
certify. Checked on the CPU against a brute-force FP64 top-k (numpy), on data with exact ties
and near-duplicates, and with a shortlist so short that most queries take the fallback."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _brute(base, queries, k):
    b = base.astype(np.float64)
    q = queries.astype(np.float64)
    d = ((q[:, None, :] - b[None, :, :]) ** 2).sum(-1)
    return np.argsort(d, axis=1, kind="stable")[:, :k], d


@pytest.mark.parametrize("shortlist", [64, 12])
def test_ground_truth_equals_brute_force(shortlist):
    import torch

    import bench

    rng = np.random.default_rng(3)
    base = rng.standard_normal((3000, 48)).astype(np.float32)
    base[100] = base[7]                      # an exact duplicate pair
    base[200] = base[9] + 1e-6               # a near-duplicate
    base[300:330] = base[55]                 # 31 copies: the query base[55] has 31 rows at distance 0
    queries = np.concatenate([rng.standard_normal((40, 48)).astype(np.float32), base[[7, 9, 55]]])
    gt, info = bench.ground_truth(torch, torch.from_numpy(base), torch.from_numpy(queries), 10, shortlist=shortlist)
    ref, d = _brute(base, queries, 10)
    got = gt.numpy()
    # the sets of the 10 nearest are equal; ids at exactly equal distances may come in either order
    for i in range(len(queries)):
        np.testing.assert_array_equal(np.sort(d[i, got[i]]), np.sort(d[i, ref[i]]))
    assert info["certified"] + info["full_fp64_scan"] == len(queries)
    if shortlist == 12:
        # no bound separates the 10th from the 12th of 31 equal distances: that query takes the fallback
        assert info["full_fp64_scan"] >= 1


def test_fp32_score_error_bound_covers_observed_errors():
    import bench

    rng = np.random.default_rng(5)
    dim = 1536
    base = rng.standard_normal((2000, dim)).astype(np.float32)
    base /= np.linalg.norm(base, axis=1, keepdims=True)
    q = rng.standard_normal(dim).astype(np.float32)
    q /= np.linalg.norm(q)
    bn32 = (base * base).sum(1, dtype=np.float32)
    e32 = bn32 - np.float32(2.0) * (base @ q)
    exact = (base.astype(np.float64) ** 2).sum(1) - 2.0 * base.astype(np.float64) @ q.astype(np.float64)
    bound = bench.fp32_score_error_bound(dim, float(np.sqrt(bn32.max())), float(np.linalg.norm(q)))
    assert np.abs(e32.astype(np.float64) - exact).max() < bound
