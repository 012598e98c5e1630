"""The GPU Vamana build (rabitq_build_vamana_graph, rabitq_bridge.cpp:224-303) against graphs the
reference itself built (tests/golden: the search fixtures' graphs and build_variants.npz) and, at
sizes past the fixtures, against the oracle's restated build. Graphs must be identical: same
degree and the same neighbour ids in the same order for every node."""
import ctypes as C

import numpy as np
import pytest

from cases import BUILD_VARIANTS, SEARCH_CASES, SEARCH_GRAPH_ARGS
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _space(g):
    from quantization_graph_gb300.space import RabitqSpace

    return RabitqSpace(int(g["dim"]), g["center"])


def _gpu_build(torch, sp, compact, **kw):
    from quantization_graph_gb300 import graph_build

    deg, edges, evals = graph_build.build_vamana(sp, torch.from_numpy(np.ascontiguousarray(compact)).cuda(), **kw)
    torch.cuda.synchronize()
    return deg.cpu().numpy().view(np.uint32), edges.cpu().numpy().view(np.uint32), evals


def _assert_same_graph(deg, edges, gdeg, gedges, what):
    mism = np.nonzero(deg != gdeg)[0]
    assert mism.size == 0, f"{what}: degree differs at {mism[:10]} ({deg[mism[:5]]} vs {gdeg[mism[:5]]})"
    for i in range(len(deg)):
        if not np.array_equal(edges[i, :deg[i]], gedges[i, :gdeg[i]]):
            raise AssertionError(f"{what}: node {i}: {edges[i, :deg[i]]} vs {gedges[i, :gdeg[i]]}")


@pytest.mark.parametrize("name", list(SEARCH_CASES))
def test_build_matches_reference_graph(cuda, name):
    g = load_golden(name)
    deg, edges, evals = _gpu_build(cuda, _space(g), g["compact"], **SEARCH_GRAPH_ARGS[name])
    _assert_same_graph(deg, edges, g["degrees"], g["edges"], name)
    assert evals > 0
    # nothing past a degree
    assert all(not edges[i, deg[i]:].any() for i in range(len(deg)))


@pytest.mark.parametrize("variant", list(BUILD_VARIANTS))
def test_build_variants_match_reference(cuda, variant):
    v = load_golden("build_variants")
    kw = dict(BUILD_VARIANTS[variant])
    g = load_golden(kw.pop("src"))
    deg, edges, _ = _gpu_build(cuda, _space(g), g["compact"], **kw)
    _assert_same_graph(deg, edges, v[f"{variant}_degrees"], v[f"{variant}_edges"], variant)


def test_bridge_entry_point_matches_reference(cuda):
    """rabitq_build_vamana_graph itself, host buffers, called as ours_diskann.rs:2096-2120 does:
    graph, sidecar, strides."""
    from quantization_graph_gb300 import _native as N

    lib = N.load()
    g = load_golden("search_c1")
    sp = _space(g)
    compact = np.ascontiguousarray(g["compact"])
    n, r = compact.shape[0], 32
    deg = np.zeros(n, np.uint32)
    edges = np.zeros(n * r, np.uint32)
    msb = np.zeros((n, g["msb"].shape[1]), np.uint8)
    factors = np.zeros((n, 20), np.uint8)
    ms, fb, ev = C.c_size_t(0), C.c_size_t(0), C.c_uint64(0)
    a = SEARCH_GRAPH_ARGS["search_c1"]
    ok = lib.rabitq_build_vamana_graph(
        sp.ptr, C.c_void_p(compact.ctypes.data), n, compact.shape[1], r, a["l_build"], C.c_float(a["alpha"]),
        a["beam"], a["batch"], a["refine"], a["cap"], a["stop_hops"], C.c_void_p(deg.ctypes.data),
        C.c_void_p(edges.ctypes.data), r, C.c_void_p(msb.ctypes.data), C.c_void_p(factors.ctypes.data),
        C.byref(ms), C.byref(fb), C.byref(ev))
    assert ok, N.last_error()
    _assert_same_graph(deg, edges.reshape(n, r), g["degrees"], g["edges"], "bridge")
    np.testing.assert_array_equal(msb, g["msb"])
    np.testing.assert_array_equal(factors, g["factors"])
    assert ms.value == g["msb"].shape[1] and fb.value == 20 and ev.value > 0
    # the reference's argument checks: edge stride below R, alpha below 1
    assert not lib.rabitq_build_vamana_graph(
        sp.ptr, C.c_void_p(compact.ctypes.data), n, compact.shape[1], r, 64, C.c_float(1.2), 1, 256, 0, 0, 0,
        C.c_void_p(deg.ctypes.data), C.c_void_p(edges.ctypes.data), r - 1, C.c_void_p(msb.ctypes.data),
        C.c_void_p(factors.ctypes.data), C.byref(ms), C.byref(fb), C.byref(ev))
    assert not lib.rabitq_build_vamana_graph(
        sp.ptr, C.c_void_p(compact.ctypes.data), n, compact.shape[1], r, 64, C.c_float(0.9), 1, 256, 0, 0, 0,
        C.c_void_p(deg.ctypes.data), C.c_void_p(edges.ctypes.data), r, C.c_void_p(msb.ctypes.data),
        C.c_void_p(factors.ctypes.data), C.byref(ms), C.byref(fb), C.byref(ev))


@pytest.mark.parametrize("case", ["c1_20k", "d960_6k", "d1536_4k"])
def test_build_matches_oracle_at_scale(cuda, oracle, case):
    """Sizes past the fixtures (several 4096-node batches, hub nodes with thousands of back-edges
    in the first batch), against the oracle's restated build."""
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.space import RabitqSpace

    if case == "c1_20k":
        X, _ = synthetic.gmm(20000, 128, components=64, sigma=0.3, seed=11)
        kw = dict(r=32, l_build=100, alpha=1.2, beam=1, batch=4096, refine=1, cap=256, stop_hops=2)
    elif case == "d960_6k":
        X = synthetic.anisotropic(6000, 960, alpha=1.2, seed=21, absolute=True)
        kw = dict(r=64, l_build=128, alpha=1.2, beam=1, batch=4096, refine=1, cap=96, stop_hops=2)
    else:
        X = synthetic.anisotropic(4000, 1536, alpha=0.8, seed=31, normalize=True)
        kw = dict(r=48, l_build=96, alpha=1.2, beam=2, batch=1500, refine=1, cap=0, stop_hops=0)
    center = X.mean(0).astype(np.float32)
    o = oracle.Oracle(X.shape[1], center)
    compact, _ = o.encode(X)
    gdeg, gedges, _ = o.build_graph(compact, **kw)
    deg, edges, _ = _gpu_build(cuda, RabitqSpace(X.shape[1], center), compact, **kw)
    _assert_same_graph(deg, edges, gdeg, gedges, case)


@pytest.mark.parametrize("name", ["edge_r16", "edge_r8_beam2", "edge_n3"])
def test_build_edge_cases_match_reference(cuda, name):
    """Duplicate / near-duplicate / zero vectors and a 3-node index on the GPU."""
    from cases import BUILD_EDGE_ARGS

    v = load_golden("build_edges")
    kw = dict(BUILD_EDGE_ARGS[name])
    n = kw.pop("n", len(v["compact"]))
    g = dict(dim=128, center=v["center"])
    deg, edges, _ = _gpu_build(cuda, _space(g), v["compact"][:n], **kw)
    _assert_same_graph(deg, edges, v[f"{name}_degrees"], v[f"{name}_edges"], name)
