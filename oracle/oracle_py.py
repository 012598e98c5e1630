"""ctypes wrappers for the test oracles (test infrastructure only).

`Oracle` wraps oracle/_build/libqg_oracle.so, the C++ restatement of the reference's query
path. `Reference` wraps oracle/_ref/libqg_ref.so, the reference's own bridge
(experiments/02_diskann_fair/native/rabitq_bridge.cpp) compiled from its sources, which
exists only on a host where the reference tree is present. Only tests/, the smoke check and
bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libqg_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libqg_ref.so")

PAPER_ESTIMATE = np.dtype(
    [("lower_bound", "<f4"), ("short_ip", "<f4"), ("alpha", "<f4"), ("ip_hat", "<f4"),
     ("error_bound", "<f4"), ("valid", "u1")], align=True)
INTERVAL = np.dtype([("estimate", "<f4"), ("lower_bound", "<f4"), ("upper_bound", "<f4")])
STATS_FIELDS = ("visited_nodes", "distance_computations", "hops", "paper_checked",
                "paper_would_prune", "paper_not_pruned", "paper_full_saved",
                "paper_msb_kernel_calls", "paper_remaining_kernel_calls")
STATS = np.dtype([(f, "<u8") for f in STATS_FIELDS])
assert PAPER_ESTIMATE.itemsize == 24 and INTERVAL.itemsize == 12


class SearchParams(C.Structure):
    _fields_ = [("k", C.c_size_t), ("l_value", C.c_size_t), ("beam_width", C.c_size_t),
                ("epsilon0", C.c_float), ("rerank_candidates", C.c_size_t),
                ("early_stop_hops", C.c_size_t), ("kth_stop", C.c_int), ("codec", C.c_int),
                ("fused_int_rerank", C.c_int)]


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when the reference tree exists, the reference bridge)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def reference_available() -> bool:
    return os.path.exists(REF_SO)


class _Lib:
    _cache: dict = {}

    @classmethod
    def load(cls, path):
        if path not in cls._cache:
            if not os.path.exists(path):
                raise FileNotFoundError(f"{path} is not built (make -C oracle)")
            cls._cache[path] = C.CDLL(path)
        return cls._cache[path]


class Oracle:
    """The restatement: one space (seed 100 by default), INT8 query codec by default (codec: 0 Full,
    1 B1, 2 Int4, 3 Int8, 4 B1Main, 5 FullStaged, 6 FullRerankScalar, 7 FullScalar)."""

    def __init__(self, dim: int, center: np.ndarray, seed: int = 100, codec: int = 3):
        self.lib = lib = _Lib.load(ORACLE_SO)
        lib.qgo_space_new.restype = C.c_void_p
        lib.qgo_space_new.argtypes = [C.c_size_t, C.c_uint32]
        for name in ("qgo_code_dim", "qgo_full_bytes", "qgo_compact_bytes", "qgo_residual_bytes",
                     "qgo_msb_bytes"):
            getattr(lib, name).restype = C.c_size_t
            getattr(lib, name).argtypes = [C.c_void_p]
        lib.qgo_space_center_norm_sqr.restype = C.c_float
        lib.qgo_space_center_norm_sqr.argtypes = [C.c_void_p]
        lib.qgo_prepared_new.restype = C.c_void_p
        lib.qgo_prepared_new.argtypes = [C.c_void_p]
        lib.qgo_dither_seed.restype = C.c_uint64
        lib.qgo_dither_seed.argtypes = [C.c_void_p, C.c_size_t, C.c_uint32]
        lib.qgo_symmetric_distance.restype = C.c_float
        lib.qgo_symmetric_distance.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        self.dim = dim
        self.space = C.c_void_p(lib.qgo_space_new(dim, seed))
        self.center = np.ascontiguousarray(center, dtype=np.float32)
        lib.qgo_space_set_center(self.space, _p(self.center))
        self.D = lib.qgo_code_dim(self.space)
        self.full_bytes = lib.qgo_full_bytes(self.space)
        self.compact_bytes = lib.qgo_compact_bytes(self.space)
        self.residual_bytes = lib.qgo_residual_bytes(self.space)
        self.msb_bytes = lib.qgo_msb_bytes(self.space)
        self.prep = C.c_void_p(lib.qgo_prepared_new(self.space))
        # 7 = FullScalar: a Rust-side switch (distance mode 3) over the Full prepared query
        if lib.qgo_space_set_query_codec(self.space, C.c_int(0 if codec == 7 else codec)) != 0:
            raise ValueError("the oracle prepares the codecs 0..6 (and FullScalar, 7)")
        self.codec = codec

    def __del__(self):
        try:
            self.lib.qgo_prepared_delete(self.prep)
            self.lib.qgo_space_delete(self.space)
        except Exception:
            pass

    def signs(self):
        out = np.empty(self.D, np.float32)
        self.lib.qgo_space_signs(self.space, _p(out))
        return out

    def rotated_center(self):
        out = np.empty(self.D, np.float32)
        self.lib.qgo_space_rotated_center(self.space, _p(out))
        return out

    def center_norm_sqr(self):
        return self.lib.qgo_space_center_norm_sqr(self.space)

    def rotate(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(self.D, np.float32)
        self.lib.qgo_rotate(self.space, _p(x), _p(out))
        return out

    def encode_full(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros(self.full_bytes, np.uint8)
        self.lib.qgo_encode_full(self.space, _p(x), _p(out))
        return out

    def encode(self, X, threads=0):
        X = np.ascontiguousarray(X, np.float32)
        n = X.shape[0]
        compact = np.zeros((n, self.compact_bytes), np.uint8)
        residual = np.zeros((n, self.residual_bytes), np.uint8)
        self.lib.qgo_encode_batch(self.space, _p(X), C.c_size_t(n), _p(compact), _p(residual),
                                  C.c_int(threads))
        return compact, residual

    def sidecar(self, compact):
        compact = np.ascontiguousarray(compact)
        n = compact.shape[0]
        msb = np.zeros((n, self.msb_bytes), np.uint8)
        factors = np.zeros((n, 20), np.uint8)
        self.lib.qgo_export_sidecar(self.space, _p(compact), C.c_size_t(n),
                                    C.c_size_t(compact.shape[1]), _p(msb), _p(factors))
        return msb, factors

    def symmetric_distance(self, a, b):
        return self.lib.qgo_symmetric_distance(self.space, _p(np.ascontiguousarray(a)),
                                               _p(np.ascontiguousarray(b)))

    def prepare(self, q):
        q = np.ascontiguousarray(q, np.float32)
        self._q = q
        self.lib.qgo_prepare(self.space, _p(q), self.prep)
        rr = np.empty(self.D, np.float32)
        codes = np.empty(self.D, np.int8)
        sc = np.empty(4, np.float32)
        cs = np.zeros(1, np.int64)
        self.lib.qgo_prepared_export(self.prep, _p(rr), _p(codes), _p(sc), _p(cs))
        out = dict(rotated_residual=rr, codes=codes, query_norm_sqr=sc[0], query_norm=sc[1],
                   half_sum=sc[2], scale=sc[3], code_sum=int(cs[0]))
        if self.codec in (1, 4):
            bits = np.zeros(self.msb_bytes, np.uint8)
            b1 = np.zeros(3, np.float32)
            ss = np.zeros(1, np.int64)
            self.lib.qgo_prepared_export_b1(self.prep, _p(bits), _p(b1), _p(ss))
            out.update(b1_bits=bits, b1_scalars=b1, b1_signed_sum=int(ss[0]))
        return out

    def dither_seed(self, q):
        q = np.ascontiguousarray(q, np.float32)
        return self.lib.qgo_dither_seed(_p(q), C.c_size_t(q.shape[0]), C.c_uint32(0))

    def dither_draws(self, seed, count):
        out = np.empty(count, np.float64)
        self.lib.qgo_dither_draws(C.c_uint64(seed), C.c_size_t(count), _p(out))
        return out

    def distance_b1(self, record):
        """query_distance_b1 (B1 / B1Main codecs) on the most recently prepared query."""
        self.lib.qgo_distance_b1.restype = C.c_float
        self.lib.qgo_distance_b1.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        return self.lib.qgo_distance_b1(self.space, self.prep, _p(np.ascontiguousarray(record)))

    # The batched kernels act on the most recently prepared query.
    def gate(self, ids, msb, factors, eps=1.9):
        ids = np.ascontiguousarray(ids, np.uint32)
        out = np.zeros(len(ids), PAPER_ESTIMATE)
        self.lib.qgo_gate_batch(self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(msb),
                                C.c_size_t(msb.shape[1]), _p(factors), C.c_size_t(factors.shape[1]),
                                C.c_float(eps), _p(out))
        return out

    def distance(self, ids, modes, records, short_ips):
        ids = np.ascontiguousarray(ids, np.uint32)
        modes = np.ascontiguousarray(modes, np.uint8)
        short_ips = np.ascontiguousarray(short_ips, np.float32)
        out = np.zeros(len(ids), np.float32)
        self.lib.qgo_distance_batch(self.space, self.prep, _p(ids), _p(modes), C.c_size_t(len(ids)),
                                    _p(records), C.c_size_t(records.shape[1]), _p(short_ips), _p(out))
        return out

    def residual(self, ids, records, residual, long_d):
        ids = np.ascontiguousarray(ids, np.uint32)
        long_d = np.ascontiguousarray(long_d, np.float32)
        out = np.zeros(len(ids), INTERVAL)
        self.lib.qgo_residual_batch(self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(records),
                                    C.c_size_t(records.shape[1]), _p(residual),
                                    C.c_size_t(residual.shape[1]), _p(long_d), _p(out))
        return out

    def search(self, queries, index, k=10, L=40, eps=1.9, rerank=100, beam=1, early_stop=0,
               kth_stop=False, threads=0, fused=False):
        """fused: the rerank of an Int8 / Int4 traversal by the fused restore + residual kernel
        (the RABITQ_ENABLE_FUSED_INT_RERANK ablation)."""
        return _search(self.lib.qgo_search_batch, [self.space], queries, index, k, L, eps,
                       rerank, beam, early_stop, kth_stop, threads, codec=self.codec, fused=fused)

    def gate_encoded(self, ids, records, eps=1.9):
        """compute_paper_prune_estimate (space_rabitq.h:3926-3959): the gate from the encoded
        records (rabitq_paper_estimate / rabitq_paper_estimate_batch)."""
        ids = np.ascontiguousarray(ids, np.uint32)
        records = np.ascontiguousarray(records)
        out = np.zeros(len(ids), PAPER_ESTIMATE)
        self.lib.qgo_gate_encoded_batch(self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(records),
                                        C.c_size_t(records.shape[1]), C.c_float(eps), _p(out))
        return out

    def full_residual(self, ids, records, residual):
        """The fused restore + residual rerank (compute_full_residual_distance_intervals_batch_by_id,
        space_rabitq.h:5557-5778) on the prepared query: [n, 3] (estimate, lower, upper)."""
        ids = np.ascontiguousarray(ids, np.uint32)
        records = np.ascontiguousarray(records)
        residual = np.ascontiguousarray(residual)
        out = np.zeros((len(ids), 3), np.float32)
        self.lib.qgo_full_residual_batch(self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(records),
                                         C.c_size_t(records.shape[1]), _p(residual),
                                         C.c_size_t(residual.shape[1]), _p(out))
        return out

    def build_graph(self, compact, r=32, l_build=100, alpha=1.2, beam=1, batch=4096, refine=1,
                    cap=256, stop_hops=2, threads=0):
        """The restated Vamana build; same arguments as Reference.build_graph.
        Returns (degrees, edges [n, r], distances evaluated)."""
        compact = np.ascontiguousarray(compact)
        n = compact.shape[0]
        degrees = np.zeros(n, np.uint32)
        edges = np.zeros((n, r), np.uint32)
        evals = C.c_uint64(0)
        rc = self.lib.qgo_build_vamana(
            self.space, _p(compact), C.c_size_t(n), C.c_size_t(compact.shape[1]), C.c_size_t(r),
            C.c_size_t(l_build), C.c_float(alpha), C.c_size_t(beam), C.c_size_t(batch), C.c_size_t(refine),
            C.c_size_t(cap), C.c_size_t(stop_hops), _p(degrees), _p(edges), C.c_size_t(r), C.byref(evals),
            C.c_int(threads))
        if rc != 0:
            raise RuntimeError("oracle graph build failed")
        return degrees, edges, int(evals.value)

    def exact_knn(self, base, queries, k, threads=0):
        base = np.ascontiguousarray(base, np.float32)
        queries = np.ascontiguousarray(queries, np.float32)
        ids = np.zeros((len(queries), k), np.uint32)
        d = np.zeros((len(queries), k), np.float64)
        self.lib.qgo_exact_knn(_p(base), C.c_size_t(len(base)), _p(queries), C.c_size_t(len(queries)),
                               C.c_size_t(base.shape[1]), C.c_size_t(k), _p(ids), _p(d), C.c_int(threads))
        return ids, d


def _search(fn, lead_args, queries, index, k, L, eps, rerank, beam, early_stop, kth_stop, threads,
            dim_arg=None, codec=3, fused=False):
    queries = np.ascontiguousarray(queries, np.float32)
    nq = queries.shape[0]
    prm = SearchParams(k, L, beam, eps, rerank, early_stop, 1 if kth_stop else 0, codec, 1 if fused else 0)
    ids = np.zeros((nq, k), np.uint32)
    dists = np.zeros((nq, k), np.float32)
    stats = np.zeros(nq, STATS)
    args = list(lead_args)
    if dim_arg is not None:
        args.append(C.c_size_t(dim_arg))
    rc = fn(*args, _p(queries), C.c_size_t(nq), C.byref(prm), _p(index["compact"]),
            C.c_size_t(index["compact"].shape[1]), _p(index["residual"]),
            C.c_size_t(index["residual"].shape[1]), _p(index["msb"]), C.c_size_t(index["msb"].shape[1]),
            _p(index["factors"]), C.c_size_t(index["factors"].shape[1]), _p(index["degrees"]),
            _p(index["edges"]), C.c_size_t(index["edges"].shape[1]),
            C.c_size_t(index["total_points"]), C.c_size_t(index["base_points"]),
            _p(ids), _p(dists), _p(stats), C.c_int(threads))
    if rc != 0:
        raise RuntimeError(f"search failed with status {rc}")
    return ids, dists, stats


class Reference:
    """The reference's own bridge (rabitq_* entry points) plus the probe accessors."""

    def __init__(self, dim: int, center: np.ndarray, seed: int = 100, codec: int = 3):
        self.lib = lib = _Lib.load(REF_SO)
        lib.rabitq_space_new.restype = C.c_void_p
        lib.rabitq_space_new.argtypes = [C.c_size_t, C.c_uint32, C.c_size_t, C.c_size_t, C.c_size_t,
                                         C.c_bool, C.c_bool]
        lib.rabitq_space_set_center.restype = C.c_bool
        lib.rabitq_space_set_center.argtypes = [C.c_void_p, C.c_void_p]
        for name in ("rabitq_full_record_bytes", "rabitq_compact_record_bytes",
                     "rabitq_residual_record_bytes", "rabitq_paper_msb_code_bytes"):
            getattr(lib, name).restype = C.c_size_t
            getattr(lib, name).argtypes = [C.c_void_p]
        lib.rabitq_prepare_query.restype = C.c_void_p
        lib.rabitq_prepare_query.argtypes = [C.c_void_p, C.c_void_p]
        lib.rabitq_symmetric_distance.restype = C.c_float
        lib.rabitq_symmetric_distance.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.rabitq_query_distance.restype = C.c_float
        lib.rabitq_query_distance.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.rabitq_build_vamana_graph.restype = C.c_bool
        self.dim = dim
        self.space = C.c_void_p(lib.rabitq_space_new(dim, seed, 1, 4, 16, True, True))
        self.center = np.ascontiguousarray(center, dtype=np.float32)
        assert lib.rabitq_space_set_center(self.space, _p(self.center))
        # native codec ids 0..6 (space_rabitq.h:36-44); 7 = FullScalar prepares as Full (ours_diskann.rs:300-310)
        lib.rabitq_set_query_coarse_codec(self.space, C.c_int(0 if codec == 7 else codec))
        self.codec = codec
        self.full_bytes = lib.rabitq_full_record_bytes(self.space)
        self.compact_bytes = lib.rabitq_compact_record_bytes(self.space)
        self.residual_bytes = lib.rabitq_residual_record_bytes(self.space)
        self.msb_bytes = lib.rabitq_paper_msb_code_bytes(self.space)
        self.D = self.msb_bytes * 8
        self.prep = None

    def __del__(self):
        try:
            self.lib.rabitq_space_delete(self.space)
        except Exception:
            pass

    def rotate(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.empty(self.D, np.float32)
        self.lib.qgref_rotate(self.space, _p(x), _p(out))
        return out

    def encode_full(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros(self.full_bytes, np.uint8)
        assert self.lib.rabitq_encode_full(self.space, _p(x), _p(out))
        return out

    def encode(self, X):
        X = np.ascontiguousarray(X, np.float32)
        n = X.shape[0]
        compact = np.zeros((n, self.compact_bytes), np.uint8)
        residual = np.zeros((n, self.residual_bytes), np.uint8)
        full = np.zeros(self.full_bytes, np.uint8)
        for i in range(n):
            self.lib.rabitq_encode_full(self.space, _p(X[i]), _p(full))
            self.lib.rabitq_copy_compact(self.space, _p(full), C.c_void_p(compact[i].ctypes.data))
            self.lib.rabitq_copy_residual_record(self.space, _p(full), C.c_void_p(residual[i].ctypes.data))
        return compact, residual

    def sidecar(self, compact):
        compact = np.ascontiguousarray(compact)
        n = compact.shape[0]
        msb = np.zeros((n, self.msb_bytes), np.uint8)
        factors = np.zeros((n, 20), np.uint8)
        assert self.lib.rabitq_export_paper_sidecar(self.space, _p(compact), C.c_size_t(n),
                                                    C.c_size_t(compact.shape[1]), _p(msb), _p(factors))
        return msb, factors

    def symmetric_distance(self, a, b):
        return self.lib.rabitq_symmetric_distance(self.space, _p(np.ascontiguousarray(a)),
                                                  _p(np.ascontiguousarray(b)))

    def prepare(self, q):
        q = np.ascontiguousarray(q, np.float32)
        self._q = q  # the prepared query keeps a pointer to the raw query
        self.prep = C.c_void_p(self.lib.rabitq_prepare_query(self.space, _p(q)))
        rr = np.empty(self.D, np.float32)
        codes = np.empty(self.D, np.int8)
        sc = np.empty(4, np.float32)
        cs = np.zeros(1, np.int64)
        self.lib.qgref_prepared_export(self.prep, C.c_size_t(self.D), _p(rr), _p(codes), _p(sc), _p(cs))
        out = dict(rotated_residual=rr, codes=codes, query_norm_sqr=sc[0], query_norm=sc[1],
                   half_sum=sc[2], scale=sc[3], code_sum=int(cs[0]))
        if self.codec in (1, 4):
            bits = np.zeros(self.msb_bytes, np.uint8)
            b1 = np.zeros(3, np.float32)
            ss = np.zeros(1, np.int64)
            self.lib.qgref_prepared_export_b1(self.prep, C.c_size_t(self.D), _p(bits), _p(b1), _p(ss))
            out.update(b1_bits=bits, b1_scalars=b1, b1_signed_sum=int(ss[0]))
        return out

    def gate(self, ids, msb, factors, eps=1.9):
        ids = np.ascontiguousarray(ids, np.uint32)
        out = np.zeros(len(ids), PAPER_ESTIMATE)
        self.lib.rabitq_paper_estimate_batch_sidecar(
            self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(msb), C.c_size_t(msb.shape[1]),
            _p(factors), C.c_size_t(factors.shape[1]), C.c_float(eps), _p(out))
        return out

    def distance(self, ids, modes, records, short_ips):
        ids = np.ascontiguousarray(ids, np.uint32)
        modes = np.ascontiguousarray(modes, np.uint8)
        short_ips = np.ascontiguousarray(short_ips, np.float32)
        out = np.zeros(len(ids), np.float32)
        self.lib.rabitq_query_distance_batch(self.space, self.prep, _p(ids), _p(modes),
                                             C.c_size_t(len(ids)), _p(records),
                                             C.c_size_t(records.shape[1]), _p(short_ips), _p(out))
        return out

    def full_residual(self, ids, records, residual):
        """rabitq_full_residual_distance_batch (the fused FP32 restore + residual rerank kernel,
        space_rabitq.h:5557-5778) on the most recently prepared query: [n, 3] (est, lo, hi)."""
        ids = np.ascontiguousarray(ids, np.uint32)
        out = np.zeros((len(ids), 3), np.float32)
        self.lib.rabitq_full_residual_distance_batch(
            self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(records), C.c_size_t(records.shape[1]),
            _p(residual), C.c_size_t(residual.shape[1]), _p(out))
        return out

    def gate_encoded(self, ids, records, eps=1.9):
        """rabitq_paper_estimate_batch: the gate from the encoded records."""
        ids = np.ascontiguousarray(ids, np.uint32)
        records = np.ascontiguousarray(records)
        out = np.zeros(len(ids), PAPER_ESTIMATE)
        self.lib.rabitq_paper_estimate_batch(self.space, self.prep, _p(ids), C.c_size_t(len(ids)), _p(records),
                                             C.c_size_t(records.shape[1]), C.c_float(eps), _p(out))
        return out

    def distance_b1(self, record):
        """rabitq_query_distance_b1 on the most recently prepared query (B1 / B1Main codecs)."""
        self.lib.rabitq_query_distance_b1.restype = C.c_float
        self.lib.rabitq_query_distance_b1.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        return self.lib.rabitq_query_distance_b1(self.space, self.prep, _p(np.ascontiguousarray(record)))

    def distance_single(self, record):
        return self.lib.rabitq_query_distance(self.space, self.prep, _p(np.ascontiguousarray(record)))

    def residual(self, ids, records, residual, long_d):
        ids = np.ascontiguousarray(ids, np.uint32)
        long_d = np.ascontiguousarray(long_d, np.float32)
        out = np.zeros(len(ids), INTERVAL)
        self.lib.rabitq_residual_distance_batch(self.space, self.prep, _p(ids), C.c_size_t(len(ids)),
                                                _p(records), C.c_size_t(records.shape[1]), _p(residual),
                                                C.c_size_t(residual.shape[1]), _p(long_d), _p(out))
        return out

    def save_state(self) -> bytes:
        """RaBitQSpace::saveState of the reference space."""
        self.lib.qgref_save_state.restype = C.c_size_t
        buf = np.zeros(1 << 22, np.uint8)
        n = self.lib.qgref_save_state(self.space, _p(buf), C.c_size_t(buf.size))
        if n == 0:
            raise RuntimeError("reference saveState failed")
        return bytes(buf[:n])

    def load_state(self, state: bytes) -> bool:
        """RaBitQSpace::loadState into the reference space; False when the reference rejects it."""
        b = np.frombuffer(state, np.uint8).copy()
        return bool(self.lib.qgref_load_state(self.space, _p(b), C.c_size_t(b.size)))

    def build_graph(self, compact, r=32, l_build=100, alpha=1.2, beam=1, batch=4096, refine=1,
                    cap=256, stop_hops=2):
        compact = np.ascontiguousarray(compact)
        n = compact.shape[0]
        degrees = np.zeros(n, np.uint32)
        edges = np.zeros((n, r), np.uint32)
        msb = np.zeros((n, self.msb_bytes), np.uint8)
        factors = np.zeros((n, 20), np.uint8)
        msb_stride = C.c_size_t(0)
        fbytes = C.c_size_t(0)
        evals = C.c_uint64(0)
        ok = self.lib.rabitq_build_vamana_graph(
            self.space, _p(compact), C.c_size_t(n), C.c_size_t(compact.shape[1]), C.c_size_t(r),
            C.c_size_t(l_build), C.c_float(alpha), C.c_size_t(beam), C.c_size_t(batch),
            C.c_size_t(refine), C.c_size_t(cap), C.c_size_t(stop_hops), _p(degrees), _p(edges),
            C.c_size_t(r), _p(msb), _p(factors), C.byref(msb_stride), C.byref(fbytes), C.byref(evals))
        if not ok:
            raise RuntimeError("reference graph build failed")
        self.last_build_evals = int(evals.value)
        return degrees, edges

    def search(self, queries, index, k=10, L=40, eps=1.9, rerank=100, beam=1, early_stop=0,
               kth_stop=False, threads=0, fused=False):
        return _search(self.lib.qgref_search_batch, [self.space], queries, index, k, L, eps, rerank,
                       beam, early_stop, kth_stop, threads, dim_arg=self.dim, codec=self.codec, fused=fused)
