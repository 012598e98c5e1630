"""GPU tests of the query codecs' variants and of the boundary's per-record paths: the Full codec
and its FullStaged / FullRerankScalar variants (entry points and whole searches), the fused and
per-record residual orders (rabitq_full_residual_distance_batch, rabitq_residual_distance_from_record,
FullRerankScalar's residual batch, the fused Int8 / Int4 rerank), and the gate from the encoded
record (rabitq_paper_estimate, _batch), against the reference's outputs in tests/golden. Kept in a
file of their own, after the Int8 path's tests."""
import ctypes as C

import numpy as np
import pytest

from cases import SEARCH_CASES, kernel_inputs
from conftest import load_golden

pytestmark = pytest.mark.gpu


def _p(a):
    return C.c_void_p(a.ctypes.data)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def stats_matrix(st):
    return st.view(np.uint64).reshape(len(st), -1)


@pytest.fixture(scope="module")
def lib(cuda):
    from quantization_graph_gb300 import _native as N

    return N.load()


def _space(lib, dim, center, codec=3):
    sp = C.c_void_p(lib.rabitq_space_new(dim, 100, 1, 4, 16, True, True))
    assert sp.value
    c = np.ascontiguousarray(center, np.float32)
    assert lib.rabitq_space_set_center(sp, _p(c))
    lib.rabitq_set_query_coarse_codec(sp, codec)
    return sp


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_fused_rerank_entry_point(lib, name):
    """rabitq_full_residual_distance_batch (the fused restore + residual rerank, in that kernel's
    product order) against the reference's outputs for every query x record."""
    from quantization_graph_gb300 import _native as N

    g = load_golden(name)
    v = load_golden("fused_rerank")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(lib, dim, g["center"])
    try:
        compact, residual = g["compact"], g["residual"]
        ids = np.arange(n, dtype=np.uint32)
        for q in range(nq):
            prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(np.ascontiguousarray(Q[q]))))
            assert prep.value
            iv = (N.DistanceInterval * n)()
            assert lib.rabitq_full_residual_distance_batch(sp, prep, _p(ids), n, _p(compact), compact.shape[1],
                                                           _p(residual), residual.shape[1], iv)
            got = np.frombuffer(bytes(iv), np.float32).reshape(n, 3)
            np.testing.assert_array_equal(bits(got), bits(v[name][q]))
            lib.rabitq_release_query(sp, prep)
    finally:
        lib.rabitq_space_delete(sp)


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_full_codec_entry_points(lib, name):
    """The Full codec: the FP32 MSB gate (rabitq_paper_estimate_batch_sidecar) and the mode-1
    distance with the gate's short ip (rabitq_query_distance_batch, all-mode-1 and mixed with
    mode 0, and rabitq_query_distance_with_paper) against the reference for every query x record."""
    from quantization_graph_gb300 import _native as N

    g = load_golden(name)
    v = load_golden("full_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(lib, dim, g["center"], 0)
    try:
        compact, msb, factors = g["compact"], g["msb"], g["factors"]
        ids = np.arange(n, dtype=np.uint32)
        for q in range(nq):
            prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(np.ascontiguousarray(Q[q]))))
            assert prep.value, N.last_error()
            est = (N.PaperEstimate * n)()
            assert lib.rabitq_paper_estimate_batch_sidecar(sp, prep, _p(ids), n, _p(msb), msb.shape[1],
                                                           _p(factors), factors.shape[1], C.c_float(1.9), est)
            got = np.frombuffer(bytes(est), np.uint8).reshape(n, -1)
            np.testing.assert_array_equal(got[:, :21], v[f"{name}_gate"][q][:, :21])
            sip = np.array([e.short_ip for e in est], np.float32)
            out = np.zeros(n, np.float32)
            mode1 = np.ones(n, np.uint8)
            assert lib.rabitq_query_distance_batch(sp, prep, _p(ids), _p(mode1), n, _p(compact),
                                                   compact.shape[1], _p(sip), _p(out))
            np.testing.assert_array_equal(bits(out), bits(v[f"{name}_dist_mode1"][q]))
            modes = (ids % 2).astype(np.uint8)  # mixed batch: odd records mode 1, even mode 0
            mixed = np.zeros(n, np.float32)
            assert lib.rabitq_query_distance_batch(sp, prep, _p(ids), _p(modes), n, _p(compact), compact.shape[1],
                                                   _p(sip), _p(mixed))
            want = np.where(modes == 1, v[f"{name}_dist_mode1"][q], g["dist_mode0"][q]).astype(np.float32)
            np.testing.assert_array_equal(bits(mixed), bits(want))
            single = np.array([lib.rabitq_query_distance_with_paper(sp, prep, C.c_void_p(compact[i].ctypes.data),
                                                                    C.c_float(sip[i])) for i in range(0, n, 7)],
                              np.float32)
            np.testing.assert_array_equal(bits(single), bits(v[f"{name}_dist_mode1"][q][::7]))
            lib.rabitq_release_query(sp, prep)
    finally:
        lib.rabitq_space_delete(sp)


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_per_record_residual_paths(lib, name):
    """The reference's per-record residual (rabitq_residual_distance_from_record, and
    rabitq_residual_distance_batch when the codec is FullRerankScalar) takes the fused kernel's
    product order; checked against the fused rerank's outputs for every query x record."""
    from quantization_graph_gb300 import _native as N

    g = load_golden(name)
    v = load_golden("fused_rerank")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    compact, residual = np.ascontiguousarray(g["compact"]), np.ascontiguousarray(g["residual"])
    ids = np.arange(n, dtype=np.uint32)
    for codec in (3, 6):
        sp = _space(lib, dim, g["center"], codec)
        try:
            for q in range(nq):
                prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(np.ascontiguousarray(Q[q]))))
                assert prep.value
                d0 = np.ascontiguousarray(g["dist_mode0"][q], np.float32)
                if codec == 3:
                    got = np.array([[x.estimate, x.lower_bound, x.upper_bound] for x in (
                        lib.rabitq_residual_distance_from_record(sp, prep, _p(compact[i]), _p(residual[i]),
                                                                 C.c_float(d0[i])) for i in range(n))], np.float32)
                else:
                    iv = (N.DistanceInterval * n)()
                    assert lib.rabitq_residual_distance_batch(sp, prep, _p(ids), n, _p(compact), compact.shape[1],
                                                              _p(residual), residual.shape[1], _p(d0), iv)
                    got = np.frombuffer(bytes(iv), np.float32).reshape(n, 3)
                np.testing.assert_array_equal(bits(got), bits(v[name][q]))
                lib.rabitq_release_query(sp, prep)
        finally:
            lib.rabitq_space_delete(sp)


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536"])
@pytest.mark.parametrize("codec", [3, 0])
def test_encoded_record_gate_entry_points(lib, name, codec):
    """rabitq_paper_estimate and rabitq_paper_estimate_batch: the gate computed from the encoded
    record (compute_paper_prune_estimate, a different bound from the sidecar gate's) against the
    reference for every query x record."""
    from quantization_graph_gb300 import _native as N

    g = load_golden(name)
    v = load_golden("encoded_gate")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    compact = np.ascontiguousarray(g["compact"])
    ids = np.arange(n, dtype=np.uint32)
    sp = _space(lib, dim, g["center"], codec)
    try:
        for q in range(nq):
            prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(np.ascontiguousarray(Q[q]))))
            assert prep.value
            est = (N.PaperEstimate * n)()
            assert lib.rabitq_paper_estimate_batch(sp, prep, _p(ids), n, _p(compact), compact.shape[1],
                                                   C.c_float(1.9), est)
            got = np.frombuffer(bytes(est), np.uint8).reshape(n, -1)
            np.testing.assert_array_equal(got[:, :21], v[f"{name}_c{codec}"][q][:, :21])
            single = np.array([np.frombuffer(bytes(lib.rabitq_paper_estimate(sp, prep, _p(compact[i]), C.c_float(1.9))),
                                             np.uint8) for i in range(0, n, 5)])
            np.testing.assert_array_equal(single[:, :21], v[f"{name}_c{codec}"][q][::5, :21])
            lib.rabitq_release_query(sp, prep)
    finally:
        lib.rabitq_space_delete(sp)


def test_fused_rerank_keeps_per_record_results(lib, oracle):
    """A record whose restore is not finite (NaN norm) keeps its own NaN interval and one with an
    infinite long scale takes the invalid-record distance, while the others are unchanged: the
    fused entry computes each record on its own, as the reference does (the oracle's fused
    restatement matches the reference library on these rows)."""
    from quantization_graph_gb300 import _native as N

    g = load_golden("kernels_d128")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    compact = np.ascontiguousarray(g["compact"]).copy()
    residual = np.ascontiguousarray(g["residual"])
    f32 = compact[:, :16].copy().view(np.float32)
    f32[3, 0], f32[9, 1] = np.nan, np.inf
    compact[:, :16] = f32.view(np.uint8)
    ids = np.arange(n, dtype=np.uint32)
    o = oracle.Oracle(dim, g["center"])
    sp = _space(lib, dim, g["center"])
    try:
        for q in range(2):
            query = np.ascontiguousarray(Q[q])
            prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(query)))
            assert prep.value
            iv = (N.DistanceInterval * n)()
            assert lib.rabitq_full_residual_distance_batch(sp, prep, _p(ids), n, _p(compact), compact.shape[1],
                                                           _p(residual), residual.shape[1], iv)
            got = np.frombuffer(bytes(iv), np.float32).reshape(n, 3)
            o.prepare(query)
            want = o.full_residual(ids, compact, residual)
            nan = np.isnan(want)
            np.testing.assert_array_equal(np.isnan(got), nan)  # NaN payloads differ between CPU and GPU
            np.testing.assert_array_equal(bits(got)[~nan], bits(want)[~nan])
            assert nan[3].all() and not nan[9].any() and nan.sum() == 3
            lib.rabitq_release_query(sp, prep)
    finally:
        lib.rabitq_space_delete(sp)


@pytest.mark.parametrize("name", list(SEARCH_CASES))
@pytest.mark.parametrize("codec", [3, 2])
def test_fused_int_rerank_search_matches_reference(cuda, name, codec):
    """Int8 / Int4 searches with the fused rerank switched on (RABITQ_ENABLE_FUSED_INT_RERANK in
    the reference) against the reference's kernels: ids, distance bits, counters."""
    torch = cuda
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden(name)
    v = load_golden("fused_rerank")
    _, Q = SEARCH_CASES[name]()
    sp = RabitqSpace(int(g["dim"]), g["center"], codec=codec)
    ix = OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    q = torch.from_numpy(Q).cuda()
    for L in (20, 40):
        r = ix.search(q, k=10, l_value=L, with_stats=True, fused_int_rerank=True)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), v[f"{name}_c{codec}_ids_L{L}"])
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(v[f"{name}_c{codec}_dists_L{L}"]))
        np.testing.assert_array_equal(stats_matrix(r.stats), v[f"{name}_c{codec}_stats_L{L}"])


@pytest.mark.parametrize("name", list(SEARCH_CASES))
@pytest.mark.parametrize("codec", [0, 5, 6])
def test_full_codec_search_matches_reference(cuda, name, codec):
    """The Full codec through the batched GPU search (FP32 gate against the MSB plane, survivors
    by the remaining bits with the gate's short ip, the rerank correcting those distances)
    against the reference's kernels: ids, distance bits, counters. FullStaged (5) searches as Full;
    FullRerankScalar (6) reranks in the per-record residual order."""
    torch = cuda
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace

    g = load_golden(name)
    v = load_golden("full_codec")
    _, Q = SEARCH_CASES[name]()
    sp = RabitqSpace(int(g["dim"]), g["center"], codec=codec)
    ix = OursIndex(sp, g["compact"], g["residual"], g["msb"], g["factors"], g["degrees"], g["edges"])
    q = torch.from_numpy(Q).cuda()
    for L in (20, 40):
        key = f"{name}_c{codec}" if f"{name}_c{codec}_ids_L{L}" in v else name
        r = ix.search(q, k=10, l_value=L, with_stats=True)
        np.testing.assert_array_equal(r.ids.cpu().numpy().astype(np.uint32), v[f"{key}_ids_L{L}"])
        np.testing.assert_array_equal(bits(r.distances.cpu().numpy()), bits(v[f"{key}_dists_L{L}"]))
        np.testing.assert_array_equal(stats_matrix(r.stats), v[f"{key}_stats_L{L}"])
