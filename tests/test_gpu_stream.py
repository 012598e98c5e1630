"""One captured CUDA graph serving uneven batches (sizes 1..max, per-query k and L) returns exactly
what the ordinary search returns; the launch-shape autotuner keeps results unchanged."""
import numpy as np
import pytest

from cases import SEARCH_CASES
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _index(torch):
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden("search_c1")
    sp = RabitqSpace(128, g["center"])
    return g, OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])


def test_graph_replay_matches_plain_search_on_uneven_batches(cuda):
    torch = cuda
    from quantization_graph_gb300.stream import GraphSearcher

    g, ix = _index(torch)
    _, Q = SEARCH_CASES["search_c1"]()
    rng = np.random.default_rng(7)
    allq = np.concatenate([Q] * 4)
    gs = GraphSearcher(ix, 128, max_batch=64, max_k=100, max_l=160)
    start = 0
    for size in (1, 64, 7, 33, 2, 64, 13):
        qb = allq[start:start + size]
        start += size
        kb = rng.choice([1, 10, 100], size=size).astype(np.int32)
        lb = rng.integers(10, 160, size=size).astype(np.int32)
        ids, dists = gs.search(torch.from_numpy(qb).cuda(), torch.from_numpy(kb).cuda(), torch.from_numpy(lb).cuda())
        gs.synchronize()
        ref = ix.search(torch.from_numpy(qb).cuda(), k=100, l_value=160, k_per_query=torch.from_numpy(kb),
                        l_per_query=torch.from_numpy(lb), with_stats=False)
        np.testing.assert_array_equal(ids.cpu().numpy().astype(np.uint32), ref.ids.cpu().numpy().astype(np.uint32))
        np.testing.assert_array_equal(dists.cpu().numpy().view(np.uint32), ref.distances.cpu().numpy().view(np.uint32))


def test_autotuner_keeps_results(cuda):
    torch = cuda
    from quantization_graph_gb300.stream import autotune

    g, ix = _index(torch)
    _, Q = SEARCH_CASES["search_c1"]()
    q = torch.from_numpy(Q).cuda()
    best, results = autotune(ix, q, k=10, l_value=40, repeats=1)
    assert best in [r[0] for r in results] and len(best) == 3
    r = ix.search(q, k=10, l_value=40)
    np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), g["ids_L40_k10"])


def test_graph_replay_with_learned_stop_matches_direct_call(cuda):
    """The captured graph with a stop model returns what the direct learned-stop call returns."""
    torch = cuda
    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.stream import GraphSearcher

    g, ix = _index(torch)
    _, cent = synthetic.gmm(1, 128, components=64, sigma=0.3, seed=11)
    tq, _ = synthetic.gmm(800, 128, sigma=0.3, seed=301, centres=cent)
    tq = torch.from_numpy(tq).cuda()
    truth = ix.search(tq, k=10, l_value=80, with_stats=False).ids.to(torch.int32)
    tr = ls.collect_traces(ix, tq, truth, k=10, l_value=80, every=4)
    model = ls.train(tr.features, tr.classifier_labels(), epochs=2, batch=4096, every=4, min_hops=8)
    _, Q = SEARCH_CASES["search_c1"]()
    q = torch.from_numpy(Q).cuda()
    gs = GraphSearcher(ix, 128, max_batch=64, max_k=10, max_l=80, model=model, threshold=0.8)
    n = q.shape[0]
    ids, dists = gs.search(q, torch.full((n,), 10, dtype=torch.int32, device="cuda"),
                           torch.full((n,), 80, dtype=torch.int32, device="cuda"))
    gs.synchronize()
    ref_ids, ref_d = ls.search(ix, q, model, 0.8, k=10, l_value=80)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(ids.cpu().numpy(), ref_ids.cpu().numpy())
    np.testing.assert_array_equal(dists.cpu().numpy().view(np.uint32), ref_d.cpu().numpy().view(np.uint32))


def test_search_pool_in_flight_matches_plain_search(cuda):
    """Several batches in flight over shared handles of one index (SearchPool, qg_index_share)
    return exactly what the ordinary search returns, batch by batch; a share searches on its own
    after the pool's handles are gone."""
    torch = cuda
    from quantization_graph_gb300.stream import SearchPool

    g, ix = _index(torch)
    _, Q = SEARCH_CASES["search_c1"]()
    rng = np.random.default_rng(9)
    sizes = [1, 64, 7, 33, 2, 64, 13, 50, 3, 64]
    bounds = np.concatenate([[0], np.cumsum(sizes)])
    allq = np.concatenate([Q] * (int(bounds[-1]) // len(Q) + 1))
    kq = rng.choice([1, 10, 100], size=bounds[-1]).astype(np.int32)
    lq = rng.integers(10, 160, size=bounds[-1]).astype(np.int32)
    hq = torch.from_numpy(allq[:bounds[-1]].copy()).pin_memory()
    hk, hl = torch.from_numpy(kq).pin_memory(), torch.from_numpy(lq).pin_memory()
    batches = [(hq[a:b], hk[a:b], hl[a:b]) for a, b in zip(bounds[:-1], bounds[1:])]
    out = torch.empty((bounds[-1], 100), dtype=torch.int32).pin_memory()
    pool = SearchPool(ix, 128, max_batch=64, max_k=100, max_l=160, inflight=3)
    lat, elapsed = pool.run(batches, out)
    assert len(lat) == len(sizes) and elapsed > 0
    for a, b in zip(bounds[:-1], bounds[1:]):
        ref = ix.search(hq[a:b].cuda(), k=100, l_value=160, k_per_query=hk[a:b], l_per_query=hl[a:b],
                        with_stats=False)
        np.testing.assert_array_equal(out[a:b].numpy().astype(np.uint32), ref.ids.cpu().numpy().astype(np.uint32))
    share = ix.share()
    del pool
    r = share.search(torch.from_numpy(Q).cuda(), k=10, l_value=40)
    np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), g["ids_L40_k10"])
