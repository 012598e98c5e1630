"""The drop-in boundary itself: the reference bridge's rabitq_* entry points of this library,
called exactly as the Rust side calls the reference's (ours_diskann.rs:45-242), against the
golden vectors the reference produced (encode, copies, sidecar, symmetric distance, the
batched gate / distance / residual kernels, the single-record restore; Int8 and Int4 query
codecs; B1Main's 4-bit x 1-bit distance; the Full codec's FP32 gate and mode-1 distance; the
fused rerank) and against the reference's sentinels for what is not built (the staged Full
variants).
rabitq_build_vamana_graph is covered by test_gpu_vamana_build.py."""
import ctypes as C

import numpy as np
import pytest

from cases import kernel_inputs
from conftest import load_golden

pytestmark = pytest.mark.gpu

KERNEL_CASES = ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536", "kernels_d128_int4",
                "kernels_d1536_int4"]


def _p(a):
    return C.c_void_p(a.ctypes.data)


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


@pytest.fixture(scope="module")
def lib(cuda):
    from quantization_graph_gb300 import _native as N

    return N.load()


def _space(lib, dim, center, codec=3):
    sp = C.c_void_p(lib.rabitq_space_new(dim, 100, 1, 4, 16, True, True))
    assert sp.value
    c = np.ascontiguousarray(center, np.float32)
    assert lib.rabitq_space_set_center(sp, _p(c))
    lib.rabitq_set_query_coarse_codec(sp, codec)  # Int8 (3), as the formal path sets it, or Int4 (2)
    return sp


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_encode_copy_sidecar_symmetric(lib, name):
    g = load_golden(name)
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    X, _ = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(lib, dim, g["center"])
    try:
        fb, cb, rb = (lib.rabitq_full_record_bytes(sp), lib.rabitq_compact_record_bytes(sp),
                      lib.rabitq_residual_record_bytes(sp))
        assert (fb, cb, rb) == (g["full"].shape[1], g["compact"].shape[1], g["residual"].shape[1])
        assert lib.rabitq_paper_msb_code_bytes(sp) == g["msb"].shape[1]
        assert lib.rabitq_paper_factor_bytes() == 20
        full = np.zeros(fb, np.uint8)
        compact = np.zeros((n, cb), np.uint8)
        residual = np.zeros((n, rb), np.uint8)
        for i in range(n):
            x = np.ascontiguousarray(X[i])
            assert lib.rabitq_encode_full(sp, _p(x), _p(full))
            np.testing.assert_array_equal(full, g["full"][i])
            assert lib.rabitq_copy_compact(sp, _p(full), C.c_void_p(compact[i].ctypes.data))
            assert lib.rabitq_copy_residual_record(sp, _p(full), C.c_void_p(residual[i].ctypes.data))
        np.testing.assert_array_equal(compact, g["compact"])
        np.testing.assert_array_equal(residual, g["residual"])
        msb = np.zeros_like(g["msb"])
        factors = np.zeros_like(g["factors"])
        assert lib.rabitq_export_paper_sidecar(sp, _p(compact), n, cb, _p(msb), _p(factors))
        np.testing.assert_array_equal(msb, g["msb"])
        np.testing.assert_array_equal(factors, g["factors"])
        m = g["symmetric"].shape[0]
        sym = np.array([[lib.rabitq_symmetric_distance(sp, C.c_void_p(compact[i].ctypes.data),
                                                       C.c_void_p(compact[j].ctypes.data)) for j in range(m)]
                        for i in range(m)], np.float32)
        np.testing.assert_array_equal(bits(sym), bits(g["symmetric"]))
    finally:
        lib.rabitq_space_delete(sp)


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_prepared_query_kernels(lib, name):
    from quantization_graph_gb300 import _native as N

    g = load_golden(name)
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(lib, dim, g["center"], int(g.get("codec", 3)))
    try:
        compact, residual, msb, factors = g["compact"], g["residual"], g["msb"], g["factors"]
        ids = np.arange(n, dtype=np.uint32)
        for q in range(nq):
            query = np.ascontiguousarray(Q[q])
            prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(query)))
            assert prep.value
            est = (N.PaperEstimate * n)()
            assert lib.rabitq_paper_estimate_batch_sidecar(sp, prep, _p(ids), n, _p(msb), msb.shape[1],
                                                           _p(factors), factors.shape[1], C.c_float(1.9), est)
            got = np.frombuffer(bytes(est), np.uint8).reshape(n, -1)
            np.testing.assert_array_equal(got[:, :21], g["gate"][q][:, :21])
            sip = np.array([e.short_ip for e in est], np.float32)
            out = np.zeros(n, np.float32)
            mode2 = np.full(n, 2, np.uint8)
            assert lib.rabitq_query_distance_batch(sp, prep, _p(ids), _p(mode2), n, _p(compact),
                                                   compact.shape[1], _p(sip), _p(out))
            np.testing.assert_array_equal(bits(out), bits(g["dist_mode2"][q]))
            d0 = np.zeros(n, np.float32)
            mode0, zero_ips = np.zeros(n, np.uint8), np.zeros(n, np.float32)
            assert lib.rabitq_query_distance_batch(sp, prep, _p(ids), _p(mode0), n, _p(compact),
                                                   compact.shape[1], _p(zero_ips), _p(d0))
            np.testing.assert_array_equal(bits(d0), bits(g["dist_mode0"][q]))
            single = np.array([lib.rabitq_query_distance(sp, prep, C.c_void_p(compact[i].ctypes.data))
                               for i in range(n)], np.float32)
            np.testing.assert_array_equal(bits(single), bits(g["dist_single"][q]))
            iv = (N.DistanceInterval * n)()
            assert lib.rabitq_residual_distance_batch(sp, prep, _p(ids), n, _p(compact), compact.shape[1],
                                                      _p(residual), residual.shape[1], _p(d0), iv)
            got_iv = np.frombuffer(bytes(iv), np.float32).reshape(n, 3)
            np.testing.assert_array_equal(bits(got_iv), bits(g["residual_iv"][q]))
            lib.rabitq_release_query(sp, prep)
    finally:
        lib.rabitq_space_delete(sp)


def test_sentinels_of_what_is_not_built(lib):
    g = load_golden("kernels_d128")
    assert not C.c_void_p(lib.rabitq_space_new(128, 100, 1, 3, 16, True, True)).value  # residual bits != 4
    sp = _space(lib, 128, g["center"])
    try:
        _, Q = kernel_inputs(128, int(g["n"]), int(g["nq"]), int(g["seed"]))
        query = np.ascontiguousarray(Q[0])
        prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(query)))
        rec = np.ascontiguousarray(g["compact"][0])
        assert np.isinf(lib.rabitq_query_distance_b1(sp, prep, _p(rec)))  # needs a B1Main prepared query
        sip = np.zeros(1, np.float32)
        out = np.zeros(1, np.float32)
        lib.rabitq_set_query_coarse_codec(sp, 0)  # a Full prepared query has no integer codes for mode 2
        prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(query)))
        assert prep.value
        one_id, one_mode2 = np.zeros(1, np.uint32), np.full(1, 2, np.uint8)
        assert lib.rabitq_query_distance_batch(sp, prep, _p(one_id), _p(one_mode2), 1,
                                               _p(g["compact"]), g["compact"].shape[1], _p(sip), _p(out))
        assert np.isinf(out[0])
        for codec in (5, 6, 0x105):  # FullStaged, FullRerankScalar, an id outside the enum: Full
            lib.rabitq_set_query_coarse_codec(sp, codec)
            assert C.c_void_p(lib.rabitq_prepare_query(sp, _p(query))).value
    finally:
        lib.rabitq_space_delete(sp)


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d1536"])
@pytest.mark.parametrize("codec", [4, 1])
def test_b1main_distance_entry_points(lib, name, codec):
    """rabitq_query_distance_b1 and its batch form with a B1Main prepared query (or a B1 one: both
    prepare the query's signs, and the reference gives the same values), against the reference's
    query_distance_b1 for every query x record."""
    g = load_golden(name)
    v = load_golden("b1main_codec")
    dim, n, nq = int(g["dim"]), int(g["n"]), int(g["nq"])
    _, Q = kernel_inputs(dim, n, nq, int(g["seed"]))
    sp = _space(lib, dim, g["center"], codec)
    try:
        compact = g["compact"]
        ids = np.arange(n, dtype=np.uint32)
        for q in range(nq):
            prep = C.c_void_p(lib.rabitq_prepare_query(sp, _p(np.ascontiguousarray(Q[q]))))
            assert prep.value
            single = np.array([lib.rabitq_query_distance_b1(sp, prep, C.c_void_p(compact[i].ctypes.data))
                               for i in range(n)], np.float32)
            np.testing.assert_array_equal(bits(single), bits(v[f"{name}_distance_b1"][q]))
            out = np.zeros(n, np.float32)
            assert lib.rabitq_query_distance_b1_batch(sp, prep, _p(ids), n, _p(compact), compact.shape[1], _p(out))
            np.testing.assert_array_equal(bits(out), bits(v[f"{name}_distance_b1"][q]))
            if codec == 4:  # B1Main gates with the FP32 Full gate (space_rabitq.h:4510-4531)
                from quantization_graph_gb300 import _native as N

                msb, factors = g["msb"], g["factors"]
                est = (N.PaperEstimate * n)()
                assert lib.rabitq_paper_estimate_batch_sidecar(sp, prep, _p(ids), n, _p(msb), msb.shape[1],
                                                               _p(factors), factors.shape[1], C.c_float(1.9), est)
                got = np.frombuffer(bytes(est), np.uint8).reshape(n, -1)
                np.testing.assert_array_equal(got[:, :21], load_golden("full_codec")[f"{name}_gate"][q][:, :21])
    finally:
        lib.rabitq_space_delete(sp)


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
