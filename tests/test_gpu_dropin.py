"""The drop-in boundary itself: the reference bridge's rabitq_* entry points of this library,
called exactly as the Rust side calls the reference's (ours_diskann.rs:45-242), against the
golden vectors the reference produced (encode, copies, sidecar, symmetric distance, the
batched gate / distance / residual kernels, the single-record restore; Int8 and Int4 query
codecs; B1Main's and B1's 4-bit x 1-bit distance) and against the reference's sentinels.
The Full codecs, the fused and per-record residual orders and the encoded-record gate are
covered by test_gpu_zz_codec_variants.py.
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
