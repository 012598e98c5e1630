"""Persistent batched GPU search against the reference's search results (ids, distance bits
and the nine OursPaperSearchStats counters, as verify_search_parity compares them,
ours_diskann.rs:1988-2066) and against the oracle on edge cases."""
import numpy as np
import pytest

from cases import SEARCH_CASES
from conftest import golden_index, load_golden

pytestmark = pytest.mark.gpu

VARIANTS = {"beam2": dict(beam_width=2, l_value=40, k=10), "kth": dict(kth_stop=True, l_value=40, k=10),
            "stall": dict(early_stop_hops=2, l_value=40, k=10), "k100": dict(l_value=40, k=100),
            "k1": dict(l_value=20, k=1)}


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def make_index(torch, g, degrees=None, edges=None, total=None):
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    sp = RabitqSpace(int(g["dim"]), g["center"])
    ix = OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"],
                   g["degrees"] if degrees is None else degrees, g["edges"] if edges is None else edges,
                   base_points=int(g["n"]), total_points=total)
    return sp, ix


def stats_matrix(st):
    return st.view(np.uint64).reshape(len(st), -1)


@pytest.mark.parametrize("name", list(SEARCH_CASES))
def test_search_matches_reference(cuda, name):
    torch = cuda
    g = load_golden(name)
    _, Q = SEARCH_CASES[name]()
    sp, ix = make_index(torch, g)
    for L in g["Ls"]:
        for k in g["ks"]:
            r = ix.search(torch.from_numpy(Q).cuda(), k=int(k), l_value=int(L))
            np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), g[f"ids_L{L}_k{k}"])
            np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(g[f"dists_L{L}_k{k}"]))
            np.testing.assert_array_equal(stats_matrix(r.stats), g[f"stats_L{L}_k{k}"])


@pytest.mark.parametrize("tag", list(VARIANTS))
def test_search_variants_match_reference(cuda, tag):
    torch = cuda
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    sp, ix = make_index(torch, g)
    r = ix.search(torch.from_numpy(Q).cuda(), **VARIANTS[tag])
    np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), g[f"ids_{tag}"])
    np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(g[f"dists_{tag}"]))
    np.testing.assert_array_equal(stats_matrix(r.stats), g[f"stats_{tag}"])


def test_uneven_per_query_k_and_l_match_oracle(cuda, oracle):
    torch = cuda
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    sp, ix = make_index(torch, g)
    rng = np.random.default_rng(5)
    ks = rng.choice([1, 10, 100], size=len(Q)).astype(np.int32)
    ls = rng.integers(5, 150, size=len(Q)).astype(np.int32)
    r = ix.search(torch.from_numpy(Q).cuda(), k=100, l_value=150, k_per_query=torch.from_numpy(ks),
                  l_per_query=torch.from_numpy(ls))
    o = oracle.Oracle(128, g["center"])
    gi = golden_index(g)
    ids = r.ids.cpu().numpy().astype(np.uint32)
    d = r.distances.cpu().numpy()
    for i in range(len(Q)):
        oi, od, os_ = o.search(Q[i:i + 1], gi, k=int(ks[i]), L=int(ls[i]))
        np.testing.assert_array_equal(ids[i, :ks[i]], oi[0])
        np.testing.assert_array_equal(bits(d[i, :ks[i]]), bits(od[0]))
        np.testing.assert_array_equal(stats_matrix(r.stats[i:i + 1]), stats_matrix(os_))
        assert (ids[i, ks[i]:] == 0xFFFFFFFF).all()


def test_duplicates_frozen_point_and_short_lists(cuda, oracle):
    """Adjacency with duplicate ids and a frozen start point appended last (adjacency [0])."""
    torch = cuda
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    n = int(g["n"])
    deg = g["degrees"].copy()
    edges = g["edges"].copy()
    for i in range(0, n, 7):
        if deg[i] >= 3:
            edges[i, 2] = edges[i, 0]   # duplicate neighbour inside one list
    deg[::11] = np.minimum(deg[::11], 1)  # very short lists
    deg = np.concatenate([deg, [1]]).astype(np.uint32)
    edges = np.concatenate([edges, np.zeros((1, edges.shape[1]), np.uint32)])
    sp, ix = make_index(torch, g, degrees=deg, edges=edges, total=n + 1)
    r = ix.search(torch.from_numpy(Q).cuda(), k=10, l_value=40)
    gi = golden_index(g)
    gi.update(degrees=deg, edges=edges, total_points=n + 1)
    oi, od, os_ = oracle.Oracle(128, g["center"]).search(Q, gi, k=10, L=40)
    np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), oi)
    np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(od))
    np.testing.assert_array_equal(stats_matrix(r.stats), stats_matrix(os_))


def test_out_of_range_neighbour_is_reported(cuda):
    torch = cuda
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    edges = g["edges"].copy()
    edges[0, 0] = 10 ** 6  # >= total points: the reference returns an error for the query
    sp, ix = make_index(torch, g, edges=edges)
    with pytest.raises(RuntimeError, match="QG_ERR_GRAPH"):
        ix.search(torch.from_numpy(Q).cuda(), k=10, l_value=40)
    # the index stays usable after the failed batch
    sp2, ix2 = make_index(torch, g)
    r = ix2.search(torch.from_numpy(Q[:4]).cuda(), k=10, l_value=40)
    np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), g["ids_L40_k10"][:4])


def test_empty_batch_and_repeated_calls(cuda):
    torch = cuda
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    sp, ix = make_index(torch, g)
    r0 = ix.search(torch.zeros((0, 128), device="cuda"), k=10, l_value=40)
    assert r0.ids.shape == (0, 10)
    # many batches through the same index exercise the visited-tag epochs
    for _ in range(5):
        r = ix.search(torch.from_numpy(Q).cuda(), k=10, l_value=40)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), g["ids_L40_k10"])


@pytest.mark.parametrize("dim", [40, 200, 400, 700])
def test_other_code_dims_match_oracle(cuda, oracle, dim):
    """The search kernel instantiations for D = 64, 256, 512 and 1024 against the oracle, on
    this library's own encode and graph (ids, distance bits, counters)."""
    torch = cuda
    from quantization_graph_gb300.graph_build import build_graph
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    rng = np.random.default_rng(dim)
    X = (rng.standard_normal((1500, dim)) * rng.uniform(0.2, 2.0, dim)).astype(np.float32)
    Q = (rng.standard_normal((20, dim)) * rng.uniform(0.2, 2.0, dim)).astype(np.float32)
    c = X.mean(0).astype(np.float32)
    sp = RabitqSpace(dim, c)
    xd = torch.from_numpy(X).cuda()
    compact, residual = sp.encode(xd)
    msb, factors = sp.export_paper_sidecar(compact)
    deg, edges = build_graph(sp, xd, compact, r=32, knn=64, alpha=1.2, reverse=32, refine_rounds=1, refine_l=64,
                             residual=residual, msb=msb, factors=factors)
    ix = OursIndex(sp, compact, residual, msb, factors, deg, edges)
    gi = dict(compact=compact.cpu().numpy(), residual=residual.cpu().numpy(), msb=msb.cpu().numpy(),
              factors=factors.cpu().numpy(), degrees=deg.cpu().numpy().view(np.uint32),
              edges=edges.cpu().numpy().view(np.uint32), total_points=1500, base_points=1500)
    o = oracle.Oracle(dim, c)
    for L, k in ((32, 10), (120, 100)):
        r = ix.search(torch.from_numpy(Q).cuda(), k=k, l_value=L)
        oi, od, os_ = o.search(Q, gi, k=k, L=L)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), oi)
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(od))
        np.testing.assert_array_equal(stats_matrix(r.stats), stats_matrix(os_))


@pytest.mark.parametrize("dim", [700, 1536])
def test_tile_shapes_match_oracle(cuda, oracle, dim):
    """Every tile shape of the gate / traversal loops (qg_index_set_tile) at D = 1024 and 2048
    returns the oracle's ids, distance bits and counters."""
    torch = cuda
    from quantization_graph_gb300 import _native as N
    from quantization_graph_gb300.graph_build import build_graph
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    rng = np.random.default_rng(dim + 7)
    X = (rng.standard_normal((1200, dim)) * rng.uniform(0.2, 2.0, dim)).astype(np.float32)
    Q = (rng.standard_normal((24, dim)) * rng.uniform(0.2, 2.0, dim)).astype(np.float32)
    c = X.mean(0).astype(np.float32)
    sp = RabitqSpace(dim, c)
    xd = torch.from_numpy(X).cuda()
    compact, residual = sp.encode(xd)
    msb, factors = sp.export_paper_sidecar(compact)
    deg, edges = build_graph(sp, xd, compact, r=32, knn=64, alpha=1.2, reverse=32, refine_rounds=1, refine_l=64,
                             residual=residual, msb=msb, factors=factors)
    ix = OursIndex(sp, compact, residual, msb, factors, deg, edges)
    gi = dict(compact=compact.cpu().numpy(), residual=residual.cpu().numpy(), msb=msb.cpu().numpy(),
              factors=factors.cpu().numpy(), degrees=deg.cpu().numpy().view(np.uint32),
              edges=edges.cpu().numpy().view(np.uint32), total_points=1200, base_points=1200)
    oi, od, os_ = oracle.Oracle(dim, c).search(Q, gi, k=10, L=48)
    lib = N.load()
    for tile in (0, 1, 2, 3, 4):
        N.check(lib.qg_index_set_tile(ix.handle, tile), "qg_index_set_tile")
        r = ix.search(torch.from_numpy(Q).cuda(), k=10, l_value=48)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), oi)
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(od))
        np.testing.assert_array_equal(stats_matrix(r.stats), stats_matrix(os_))
    assert lib.qg_index_set_tile(ix.handle, 5) != 0


def test_int4_codec_search_matches_reference(cuda):
    """The Int4 query codec (an ablation in the reference: scale max/8, codes in [-8, 7], the
    second dither draw) through the batched GPU search, against the reference's own kernels."""
    torch = cuda
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden("search_c1")
    v = load_golden("search_c1_int4")
    _, Q = SEARCH_CASES["search_c1"]()
    sp = RabitqSpace(128, g["center"], codec=2)
    ix = OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    q = torch.from_numpy(Q).cuda()
    for L in (20, 40, 80):
        r = ix.search(q, k=10, l_value=L, with_stats=True)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), v[f"ids_L{L}"])
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(v[f"dists_L{L}"]))
        np.testing.assert_array_equal(stats_matrix(r.stats), v[f"stats_L{L}"])


def test_b1_codec_search_matches_reference(cuda):
    """The B1 query codec through the batched GPU search (popcount gate, FP32-restore survivors)
    against the reference's own kernels with codec 1: ids, distance bits and the counters."""
    torch = cuda
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden("search_c1")
    v = load_golden("b1_codec")
    _, Q = SEARCH_CASES["search_c1"]()
    sp = RabitqSpace(128, g["center"], codec=1)
    ix = OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    q = torch.from_numpy(Q).cuda()
    for L in (20, 40, 80):
        r = ix.search(q, k=10, l_value=L, with_stats=True)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), v[f"search_c1_ids_L{L}"])
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(v[f"search_c1_dists_L{L}"]))
        np.testing.assert_array_equal(stats_matrix(r.stats), v[f"search_c1_stats_L{L}"])


@pytest.mark.parametrize("name", ["search_c1", "search_c2"])
def test_b1main_codec_search_matches_reference(cuda, name):
    """The B1Main codec (no gate; every fresh neighbour by the 4-bit x 1-bit distance) through the
    batched GPU search, against the reference: ids, distance bits, counters."""
    torch = cuda
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden(name)
    v = load_golden("b1main_codec")
    _, Q = SEARCH_CASES[name]()
    sp = RabitqSpace(int(g["dim"]), g["center"], codec=4)
    ix = OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    q = torch.from_numpy(Q).cuda()
    for L in (20, 40, 80):
        r = ix.search(q, k=10, l_value=L, with_stats=True)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), v[f"{name}_ids_L{L}"])
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(v[f"{name}_dists_L{L}"]))
        np.testing.assert_array_equal(stats_matrix(r.stats), v[f"{name}_stats_L{L}"])
