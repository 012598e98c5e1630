"""The oracle (C++ restatement) against golden vectors produced by the reference itself.

Everything here is bit-exact: codes, records, sidecars, INT8 query codes, every float of the
gate / traversal / restore / residual kernels, and search ids, distances and counters.
"""
import numpy as np
import pytest

from cases import SEARCH_CASES, kernel_inputs
from conftest import golden_index, load_golden, sha

KERNEL_CASES = ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536", "kernels_d128_int4",
                "kernels_d1536_int4"]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_kernels_bit_exact(oracle, name):
    g = load_golden(name)
    dim, n, nq, seed = int(g["dim"]), int(g["n"]), int(g["nq"]), int(g["seed"])
    X, Q = kernel_inputs(dim, n, nq, seed)
    assert sha(X) == str(g["x_sha"]) and sha(Q) == str(g["q_sha"]), "input generator drifted"
    o = oracle.Oracle(dim, g["center"], codec=int(g.get("codec", 3)))
    full = np.stack([o.encode_full(x) for x in X])
    np.testing.assert_array_equal(full, g["full"])
    compact, residual = o.encode(X)
    np.testing.assert_array_equal(compact, g["compact"])
    np.testing.assert_array_equal(residual, g["residual"])
    msb, factors = o.sidecar(g["compact"])
    np.testing.assert_array_equal(msb, g["msb"])
    np.testing.assert_array_equal(factors, g["factors"])
    ids = np.arange(n, dtype=np.uint32)
    for qi in range(nq):
        p = o.prepare(Q[qi])
        np.testing.assert_array_equal(bits(p["rotated_residual"]), bits(g["rotated_residual"][qi]))
        np.testing.assert_array_equal(p["codes"], g["codes"][qi])
        sc = np.array([p["query_norm_sqr"], p["query_norm"], p["half_sum"], p["scale"]], np.float32)
        np.testing.assert_array_equal(bits(sc), bits(g["scalars"][qi]))
        assert p["code_sum"] == int(g["code_sum"][qi])
        est = o.gate(ids, g["msb"], g["factors"])
        np.testing.assert_array_equal(est.view(np.uint8).reshape(n, -1)[:, :21], g["gate"][qi][:, :21])
        sip = est["short_ip"]
        d2 = o.distance(ids, np.full(n, 2, np.uint8), g["compact"], sip)
        np.testing.assert_array_equal(bits(d2), bits(g["dist_mode2"][qi]))
        d0 = o.distance(ids, np.zeros(n, np.uint8), g["compact"], np.zeros(n, np.float32))
        np.testing.assert_array_equal(bits(d0), bits(g["dist_mode0"][qi]))
        np.testing.assert_array_equal(bits(d0), bits(g["dist_single"][qi]))
        iv = o.residual(ids, g["compact"], g["residual"], d0)
        np.testing.assert_array_equal(bits(iv.view(np.float32).reshape(n, 3)), bits(g["residual_iv"][qi]))
    m = g["symmetric"].shape[0]
    sym = np.array([[o.symmetric_distance(g["compact"][i], g["compact"][j]) for j in range(m)] for i in range(m)],
                   np.float32)
    np.testing.assert_array_equal(bits(sym), bits(g["symmetric"]))


@pytest.mark.parametrize("name", list(SEARCH_CASES))
def test_search_loop_bit_exact(oracle, name):
    g = load_golden(name)
    X, Q = SEARCH_CASES[name]()
    assert sha(X) == str(g["x_sha"]) and sha(Q) == str(g["q_sha"])
    o = oracle.Oracle(int(g["dim"]), g["center"])
    index = golden_index(g)
    for L in g["Ls"]:
        for k in g["ks"]:
            ids, dists, stats = o.search(Q, index, k=int(k), L=int(L))
            np.testing.assert_array_equal(ids, g[f"ids_L{L}_k{k}"])
            np.testing.assert_array_equal(bits(dists), bits(g[f"dists_L{L}_k{k}"]))
            np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), g[f"stats_L{L}_k{k}"])


VARIANTS = {"beam2": dict(beam=2, L=40, k=10), "kth": dict(kth_stop=True, L=40, k=10),
            "stall": dict(early_stop=2, L=40, k=10), "k100": dict(L=40, k=100), "k1": dict(L=20, k=1)}


@pytest.mark.parametrize("tag", list(VARIANTS))
def test_search_variants_bit_exact(oracle, tag):
    g = load_golden("search_c1")
    _, Q = SEARCH_CASES["search_c1"]()
    o = oracle.Oracle(128, g["center"])
    ids, dists, stats = o.search(Q, golden_index(g), **VARIANTS[tag])
    np.testing.assert_array_equal(ids, g[f"ids_{tag}"])
    np.testing.assert_array_equal(bits(dists), bits(g[f"dists_{tag}"]))
    np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), g[f"stats_{tag}"])


def test_golden_recall_is_sane():
    g = load_golden("search_c1")
    ids = g["ids_L40_k10"]
    rec = np.mean([len(set(a) & set(b[:10])) / 10 for a, b in zip(ids, g["gt"])])
    assert rec > 0.9


def test_dither_seed_is_fnv1a(oracle):
    q = np.linspace(-1, 1, 37).astype(np.float32)
    o = oracle.Oracle(37, np.zeros(37, np.float32))
    h = 1469598103934665603
    for b in q.tobytes():
        h ^= b
        h = (h * 1099511628211) & (2 ** 64 - 1)
    h ^= (0x9E3779B97F4A7C15 + ((h << 6) & (2 ** 64 - 1)) + (h >> 2)) & (2 ** 64 - 1)
    assert o.dither_seed(q) == h
    u = o.dither_draws(12345, 1000)
    assert (u >= 0).all() and (u < 1).all()


def test_reference_cross_check_random(oracle):
    """When the reference library is present, compare on fresh random inputs too."""
    if not oracle.reference_available():
        pytest.skip("reference tree not present on this host")
    rng = np.random.default_rng(99)
    for dim in (64, 200, 1000):
        X = (rng.standard_normal((40, dim)) * rng.uniform(0.1, 3, dim)).astype(np.float32)
        c = X.mean(0).astype(np.float32)
        o, r = oracle.Oracle(dim, c), oracle.Reference(dim, c)
        np.testing.assert_array_equal(np.stack([o.encode_full(x) for x in X]), np.stack([r.encode_full(x) for x in X]))
        po, pr = o.prepare(X[0] * 1.3), r.prepare(X[0] * 1.3)
        np.testing.assert_array_equal(po["codes"], pr["codes"])


def _graph_equal(deg, edges, gdeg, gedges):
    np.testing.assert_array_equal(deg, gdeg)
    for i in range(len(deg)):
        np.testing.assert_array_equal(edges[i, :deg[i]], gedges[i, :gdeg[i]])


@pytest.mark.parametrize("name", list(SEARCH_CASES))
def test_vamana_build_matches_reference_graph(oracle, name):
    """The restated build reproduces the graph the reference's rabitq_build_vamana_graph made
    for the search fixtures (formal arguments: alpha 1.2, refine 1, cap 256, stop 2)."""
    from cases import SEARCH_GRAPH_ARGS

    g = load_golden(name)
    o = oracle.Oracle(int(g["dim"]), g["center"])
    deg, edges, _ = o.build_graph(g["compact"], **SEARCH_GRAPH_ARGS[name])
    _graph_equal(deg, edges, g["degrees"], g["edges"])


def test_vamana_build_variants_match_reference(oracle):
    """Other argument sets (beam 2-3, alpha 1.0 / 1.3 / 2.0, caps below L, no cap, several
    refinement passes, batch 1, 960-d) against the reference's own graphs, including the
    reference's distance-evaluation count."""
    from cases import BUILD_VARIANTS

    v = load_golden("build_variants")
    for name, kw in BUILD_VARIANTS.items():
        kw = dict(kw)
        g = load_golden(kw.pop("src"))
        o = oracle.Oracle(int(g["dim"]), g["center"])
        deg, edges, evals = o.build_graph(g["compact"], **kw)
        _graph_equal(deg, edges, v[f"{name}_degrees"], v[f"{name}_edges"])
        assert evals == int(v[f"{name}_evals"]), name


def test_search_loop_int4_bit_exact(oracle):
    """The Int4 query codec (scale max/8, codes in [-8, 7], the second dither draw) through the
    whole search, against the reference's own kernels with codec 2."""
    g = load_golden("search_c1")
    v = load_golden("search_c1_int4")
    _, Q = SEARCH_CASES["search_c1"]()
    o = oracle.Oracle(128, g["center"], codec=2)
    for L in (20, 40, 80):
        ids, dists, stats = o.search(Q, golden_index(g), k=10, L=L, eps=1.9, rerank=100)
        np.testing.assert_array_equal(ids, v[f"ids_L{L}"])
        np.testing.assert_array_equal(bits(dists), bits(v[f"dists_L{L}"]))
        np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), v[f"stats_L{L}"])


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d1536"])
def test_b1_codec_prepare_and_gate_bit_exact(oracle, name):
    """The B1 codec: sign bits, the 1-bit estimator's scales and the B1 gate (popcount, then the
    bound with the query's error term added) against the reference with codec 1."""
    g = load_golden(name)
    v = load_golden("b1_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    o = oracle.Oracle(dim, g["center"], codec=1)
    ids = np.arange(n, dtype=np.uint32)
    for qi in range(nq):
        p = o.prepare(Q[qi])
        np.testing.assert_array_equal(p["b1_bits"], v[f"{name}_bits"][qi])
        np.testing.assert_array_equal(bits(p["b1_scalars"]), bits(v[f"{name}_scalars"][qi]))
        assert p["b1_signed_sum"] == int(v[f"{name}_signed_sum"][qi])
        est = o.gate(ids, g["msb"], g["factors"])
        np.testing.assert_array_equal(est.view(np.uint8).reshape(n, -1)[:, :21], v[f"{name}_gate"][qi][:, :21])


def test_b1_codec_search_bit_exact(oracle):
    g = load_golden("search_c1")
    v = load_golden("b1_codec")
    _, Q = SEARCH_CASES["search_c1"]()
    o = oracle.Oracle(128, g["center"], codec=1)
    for L in (20, 40, 80):
        ids, dists, stats = o.search(Q, golden_index(g), k=10, L=L, eps=1.9, rerank=100)
        np.testing.assert_array_equal(ids, v[f"search_c1_ids_L{L}"])
        np.testing.assert_array_equal(bits(dists), bits(v[f"search_c1_dists_L{L}"]))
        np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), v[f"search_c1_stats_L{L}"])


@pytest.mark.parametrize("name", ["edge_r16", "edge_r8_beam2", "edge_n3"])
def test_vamana_build_edge_cases_match_reference(oracle, name):
    """Duplicates, near-duplicates and zero vectors (ties, zero and invalid distances) and a
    3-node index, against the reference's graphs."""
    from cases import BUILD_EDGE_ARGS, build_edge_data

    v = load_golden("build_edges")
    X = build_edge_data()
    kw = dict(BUILD_EDGE_ARGS[name])
    n = kw.pop("n", len(X))
    o = oracle.Oracle(128, v["center"])
    compact, _ = o.encode(X)
    np.testing.assert_array_equal(compact, v["compact"])
    deg, edges, _ = o.build_graph(compact[:n], **kw)
    _graph_equal(deg, edges, v[f"{name}_degrees"], v[f"{name}_edges"])


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d1536"])
def test_b1main_distance_bit_exact(oracle, name):
    """query_distance_b1 (the 4-bit data x 1-bit query estimator) for every query x record."""
    g = load_golden(name)
    v = load_golden("b1main_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    o = oracle.Oracle(dim, g["center"], codec=4)
    for qi in range(nq):
        o.prepare(Q[qi])
        d = np.array([o.distance_b1(g["compact"][i]) for i in range(n)], np.float32)
        np.testing.assert_array_equal(bits(d), bits(v[f"{name}_distance_b1"][qi]))


@pytest.mark.parametrize("name", ["search_c1", "search_c2"])
def test_b1main_search_bit_exact(oracle, name):
    """The B1Main loop (no gate, every fresh neighbour scored) against the reference's kernels."""
    g = load_golden(name)
    v = load_golden("b1main_codec")
    _, Q = SEARCH_CASES[name]()
    o = oracle.Oracle(int(g["dim"]), g["center"], codec=4)
    for L in (20, 40, 80):
        ids, dists, stats = o.search(Q, golden_index(g), k=10, L=L, eps=1.9, rerank=100)
        np.testing.assert_array_equal(ids, v[f"{name}_ids_L{L}"])
        np.testing.assert_array_equal(bits(dists), bits(v[f"{name}_dists_L{L}"]))
        np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), v[f"{name}_stats_L{L}"])


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_full_codec_gate_and_mode1_bit_exact(oracle, name):
    """The Full codec: the FP32 masked gate (16 lanes over dimensions, the reduce tree) and the
    mode-1 distance (remaining bits, the gate's short ip reused) against the reference."""
    g = load_golden(name)
    v = load_golden("full_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    o = oracle.Oracle(dim, g["center"], codec=0)
    ids = np.arange(n, dtype=np.uint32)
    for qi in range(nq):
        o.prepare(Q[qi])
        est = o.gate(ids, g["msb"], g["factors"])
        np.testing.assert_array_equal(est.view(np.uint8).reshape(n, -1)[:, :21], v[f"{name}_gate"][qi][:, :21])
        d1 = o.distance(ids, np.full(n, 1, np.uint8), g["compact"], est["short_ip"])
        np.testing.assert_array_equal(bits(d1), bits(v[f"{name}_dist_mode1"][qi]))


@pytest.mark.parametrize("name", ["search_c1", "search_c2", "search_c3"])
def test_full_codec_search_bit_exact(oracle, name):
    g = load_golden(name)
    v = load_golden("full_codec")
    _, Q = SEARCH_CASES[name]()
    o = oracle.Oracle(int(g["dim"]), g["center"], codec=0)
    for L in (20, 40):
        ids, dists, stats = o.search(Q, golden_index(g), k=10, L=L, eps=1.9, rerank=100)
        np.testing.assert_array_equal(ids, v[f"{name}_ids_L{L}"])
        np.testing.assert_array_equal(bits(dists), bits(v[f"{name}_dists_L{L}"]))
        np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), v[f"{name}_stats_L{L}"])


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_fused_rerank_bit_exact(oracle, name):
    """The fused restore + residual rerank (rabitq_full_residual_distance_batch) against the
    reference's outputs for every query x record. Its long distance is the FP32 restore's; its
    residual contracts the other product of each code pair, so on rare records it differs by one
    ulp from restore-then-residual (the path of the default rerank), which is checked too."""
    g = load_golden(name)
    v = load_golden("fused_rerank")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    o = oracle.Oracle(dim, g["center"])
    ids = np.arange(n, dtype=np.uint32)
    unfused_differs = 0
    for qi in range(nq):
        o.prepare(Q[qi])
        iv = o.full_residual(ids, g["compact"], g["residual"])
        np.testing.assert_array_equal(bits(iv), bits(v[name][qi]))
        d0 = o.distance(ids, np.zeros(n, np.uint8), g["compact"], np.zeros(n, np.float32))
        iv0 = o.residual(ids, g["compact"], g["residual"], d0).view(np.float32).reshape(n, 3)
        unfused_differs += int((bits(iv0) != bits(iv)).any(1).sum())
        assert np.all(np.abs(iv0.astype(np.float64) - iv) <= np.spacing(np.abs(iv)) * 1.01)
    if name == "kernels_d128":
        assert unfused_differs > 0  # the fixture holds a record where the two orders part


@pytest.mark.parametrize("name", ["search_c1", "search_c2", "search_c3"])
@pytest.mark.parametrize("codec", [3, 2])
def test_fused_rerank_search_bit_exact(oracle, name, codec):
    """Int8 / Int4 searches with the fused rerank switched on (RABITQ_ENABLE_FUSED_INT_RERANK,
    ours_diskann.rs:1831-1848) against the reference's kernels: same traversal, the rerank by
    rabitq_full_residual_distance_batch."""
    g = load_golden(name)
    v = load_golden("fused_rerank")
    _, Q = SEARCH_CASES[name]()
    o = oracle.Oracle(int(g["dim"]), g["center"], codec=codec)
    for L in (20, 40):
        ids, dists, stats = o.search(Q, golden_index(g), k=10, L=L, eps=1.9, rerank=100, fused=True)
        np.testing.assert_array_equal(ids, v[f"{name}_c{codec}_ids_L{L}"])
        np.testing.assert_array_equal(bits(dists), bits(v[f"{name}_c{codec}_dists_L{L}"]))
        np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), v[f"{name}_c{codec}_stats_L{L}"])


@pytest.mark.parametrize("name", ["search_c1", "search_c2", "search_c3"])
@pytest.mark.parametrize("codec", [5, 6, 7])
def test_full_codec_variants_search_bit_exact(oracle, name, codec):
    """FullStaged (5) and FullScalar (7, a Rust-side switch: distance mode 3 over a Full prepared
    query) search as Full does; FullRerankScalar (6) reranks through the bridge's per-record
    residual path (rabitq_bridge.cpp:987-1040). Against the reference's kernels."""
    g = load_golden(name)
    v = load_golden("full_codec")
    _, Q = SEARCH_CASES[name]()
    o = oracle.Oracle(int(g["dim"]), g["center"], codec=codec)
    for L in (20, 40):
        key = f"{name}_c{codec}" if f"{name}_c{codec}_ids_L{L}" in v else name
        ids, dists, stats = o.search(Q, golden_index(g), k=10, L=L, eps=1.9, rerank=100)
        np.testing.assert_array_equal(ids, v[f"{key}_ids_L{L}"])
        np.testing.assert_array_equal(bits(dists), bits(v[f"{key}_dists_L{L}"]))
        np.testing.assert_array_equal(stats.view(np.uint64).reshape(len(Q), -1), v[f"{key}_stats_L{L}"])


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536"])
@pytest.mark.parametrize("codec", [3, 0])
def test_encoded_record_gate_bit_exact(oracle, name, codec):
    """compute_paper_prune_estimate (rabitq_paper_estimate / rabitq_paper_estimate_batch): the gate
    from the encoded record, a different bound from the sidecar gate's, against the reference."""
    g = load_golden(name)
    v = load_golden("encoded_gate")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    o = oracle.Oracle(dim, g["center"], codec=codec)
    ids = np.arange(n, dtype=np.uint32)
    for qi in range(nq):
        o.prepare(Q[qi])
        est = o.gate_encoded(ids, g["compact"])
        np.testing.assert_array_equal(est.view(np.uint8).reshape(n, -1)[:, :21], v[f"{name}_c{codec}"][qi][:, :21])


def edge_gate_inputs():
    """kernels_d128 with every third sidecar factor row marked invalid (values left in place) and
    degenerate record headers: zero / negative / NaN norms, zero / NaN / infinite short scales."""
    g = load_golden("kernels_d128")
    rec = np.ascontiguousarray(g["compact"]).copy()
    fac = np.ascontiguousarray(g["factors"]).copy()
    fac[::3, 16] = 0
    f32 = rec[:, :16].copy().view(np.float32)
    f32[1, 0], f32[4, 0], f32[7, 0] = 0.0, -1.0, np.nan
    f32[10, 2], f32[13, 2], f32[16, 2] = 0.0, np.nan, np.inf
    rec[:, :16] = f32.view(np.uint8)
    return g, rec, fac


@pytest.mark.parametrize("codec", [3, 0, 1])
def test_gates_on_invalid_and_degenerate_rows_match_reference(oracle, codec):
    """The sidecar gate and the encoded-record gate on invalid factors and degenerate records,
    oracle against the reference library (where it is built)."""
    if not oracle.reference_available():
        pytest.skip("reference tree not present on this host")
    g, rec, fac = edge_gate_inputs()
    n = int(g["n"])
    _, Q = kernel_inputs(int(g["dim"]), n, int(g["nq"]), int(g["seed"]))
    ids = np.arange(n, dtype=np.uint32)
    o, r = oracle.Oracle(int(g["dim"]), g["center"], codec=codec), oracle.Reference(int(g["dim"]), g["center"], codec=codec)
    for q in range(4):
        o.prepare(Q[q])
        r.prepare(Q[q])
        for fo, fr in ((o.gate(ids, g["msb"], fac), r.gate(ids, g["msb"], fac)),
                       (o.gate_encoded(ids, rec), r.gate_encoded(ids, rec))):
            np.testing.assert_array_equal(fo.view(np.uint8).reshape(n, -1)[:, :21],
                                          fr.view(np.uint8).reshape(n, -1)[:, :21])


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
@pytest.mark.parametrize("codec", [4, 5, 6])
def test_other_codecs_gate_with_the_full_gate(oracle, name, codec):
    """compute_paper_prune_estimate_sidecar sends every codec but B1, Int4 and Int8 to the FP32 Full
    gate (space_rabitq.h:4510-4531): a B1Main or Full-variant prepared query gates as Full does
    (the reference's outputs for those codecs equal full_codec.npz's gates)."""
    g = load_golden(name)
    v = load_golden("full_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    o = oracle.Oracle(dim, g["center"], codec=codec)
    ids = np.arange(n, dtype=np.uint32)
    for qi in range(nq):
        o.prepare(Q[qi])
        est = o.gate(ids, g["msb"], g["factors"])
        np.testing.assert_array_equal(est.view(np.uint8).reshape(n, -1)[:, :21], v[f"{name}_gate"][qi][:, :21])
        if oracle.reference_available():
            r = oracle.Reference(dim, g["center"], codec=codec)
            r.prepare(Q[qi])
            np.testing.assert_array_equal(r.gate(ids, g["msb"], g["factors"]).view(np.uint8).reshape(n, -1)[:, :21],
                                          v[f"{name}_gate"][qi][:, :21])
