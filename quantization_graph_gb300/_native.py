"""Loads libqgraph_gb300.so (built in-tree by quantization_graph_gb300/build.py) and declares
the C ABI of include/qgraph_gb300.h for ctypes.

There is no CPU fallback: if the library is missing or no CUDA device is present, loading
raises, and every search/encode call fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

QG_OK = 0
QG_NOALLOC_SCRATCH_BYTES = 64 << 20  # include/qgraph_gb300.h
STATUS_NAMES = {0: "QG_OK", 1: "QG_ERR_INVALID", 2: "QG_ERR_CUDA", 3: "QG_ERR_OOM", 4: "QG_ERR_GRAPH",
                5: "QG_ERR_TIMEOUT", 6: "QG_ERR_UNSUPPORTED"}

P = C.c_void_p
SZ = C.c_size_t


class SearchParams(C.Structure):
    """qg_search_params"""
    _fields_ = [("k", C.c_int), ("l_value", C.c_int), ("beam_width", C.c_int), ("epsilon0", C.c_float),
                ("rerank_candidates", C.c_int), ("early_stop_hops", C.c_int), ("kth_stop", C.c_int),
                ("fused_int_rerank", C.c_int)]


class PaperEstimate(C.Structure):
    """RabitqPaperEstimate (rabitq_bridge.cpp:21-28)"""
    _fields_ = [("lower_bound", C.c_float), ("short_ip", C.c_float), ("alpha", C.c_float),
                ("ip_hat", C.c_float), ("error_bound", C.c_float), ("valid", C.c_uint8)]


class DistanceInterval(C.Structure):
    """RabitqDistanceInterval (rabitq_bridge.cpp:15-19)"""
    _fields_ = [("estimate", C.c_float), ("lower_bound", C.c_float), ("upper_bound", C.c_float)]


class StopModel(C.Structure):
    """qg_stop_model"""
    _fields_ = [("d_weights", C.c_void_p), ("d_norm", C.c_void_p), ("threshold", C.c_float), ("every", C.c_int),
                ("min_hops", C.c_int), ("kind", C.c_int), ("budget_scale", C.c_float), ("predict_once", C.c_int)]


class TraceRequest(C.Structure):
    """qg_trace_request"""
    _fields_ = [("d_truth", C.c_void_p), ("truth_k", C.c_int), ("every", C.c_int), ("cap", C.c_int),
                ("d_features", C.c_void_p), ("d_labels", C.c_void_p), ("d_counts", C.c_void_p)]


MLP_PARAMS = 4801

STATS_FIELDS = ("visited_nodes", "distance_computations", "hops", "paper_checked", "paper_would_prune",
                "paper_not_pruned", "paper_full_saved", "paper_msb_kernel_calls",
                "paper_remaining_kernel_calls")

# name -> (restype, argtypes)
_SIGS = {
    "rabitq_space_new": (P, [SZ, C.c_uint32, SZ, SZ, SZ, C.c_bool, C.c_bool]),
    "rabitq_space_delete": (None, [P]),
    "rabitq_space_set_center": (C.c_bool, [P, P]),
    "rabitq_space_set_centroids": (C.c_bool, [P, P, SZ]),
    "rabitq_train_centroids": (C.c_bool, [P, SZ, SZ, SZ, SZ, C.c_uint32, C.c_int, P]),
    "rabitq_full_record_bytes": (SZ, [P]),
    "rabitq_compact_record_bytes": (SZ, [P]),
    "rabitq_residual_record_bytes": (SZ, [P]),
    "rabitq_residual_block_size": (SZ, [P]),
    "rabitq_residual_bits": (SZ, [P]),
    "rabitq_encode_full": (C.c_bool, [P, P, P]),
    "rabitq_copy_compact": (C.c_bool, [P, P, P]),
    "rabitq_copy_residual_record": (C.c_bool, [P, P, P]),
    "rabitq_build_vamana_graph": (C.c_bool, [P, P, SZ, SZ, SZ, SZ, C.c_float, SZ, SZ, SZ, SZ, SZ, P, P, SZ,
                                             P, P, P, P, P]),
    "rabitq_paper_msb_code_bytes": (SZ, [P]),
    "rabitq_paper_factor_bytes": (SZ, []),
    "rabitq_export_paper_sidecar": (C.c_bool, [P, P, SZ, SZ, P, P]),
    "rabitq_symmetric_distance": (C.c_float, [P, P, P]),
    "rabitq_prepare_query": (P, [P, P]),
    "rabitq_set_query_coarse_codec": (None, [P, C.c_int]),
    "rabitq_release_query": (None, [P, P]),
    "rabitq_query_distance": (C.c_float, [P, P, P]),
    "rabitq_query_distance_b1": (C.c_float, [P, P, P]),
    "rabitq_query_distance_b1_batch": (C.c_bool, [P, P, P, SZ, P, SZ, P]),
    "rabitq_paper_estimate": (PaperEstimate, [P, P, P, C.c_float]),
    "rabitq_paper_estimate_sidecar": (PaperEstimate, [P, P, P, P, C.c_float]),
    "rabitq_paper_estimate_codec": (PaperEstimate, [P, P, P, P, P, C.c_float]),
    "rabitq_paper_estimate_codec_batch": (C.c_bool, [P, P, P, SZ, P, SZ, P, SZ, P, SZ, C.c_float, P]),
    "rabitq_query_distance_with_paper": (C.c_float, [P, P, P, C.c_float]),
    "rabitq_query_distance_with_quantized_paper": (C.c_float, [P, P, P, C.c_float]),
    "rabitq_residual_distance": (DistanceInterval, [P, P, P, C.c_float]),
    "rabitq_residual_distance_from_record": (DistanceInterval, [P, P, P, P, C.c_float]),
    "rabitq_paper_estimate_batch": (C.c_bool, [P, P, P, SZ, P, SZ, C.c_float, P]),
    "rabitq_paper_estimate_batch_sidecar": (C.c_bool, [P, P, P, SZ, P, SZ, P, SZ, C.c_float, P]),
    "rabitq_query_distance_batch": (C.c_bool, [P, P, P, P, SZ, P, SZ, P, P]),
    "rabitq_residual_distance_batch": (C.c_bool, [P, P, P, SZ, P, SZ, P, SZ, P, P]),
    "rabitq_full_residual_distance_batch": (C.c_bool, [P, P, P, SZ, P, SZ, P, SZ, P]),
    "qg_last_error": (C.c_char_p, []),
    "qg_device_sm_count": (C.c_int, []),
    "qg_index_upload_host": (C.c_int, [P, P, SZ, P, SZ, P, SZ, P, SZ, P, P, SZ, SZ, SZ, P]),
    "qg_index_upload_device": (C.c_int, [P, P, SZ, P, SZ, P, SZ, P, SZ, P, P, SZ, SZ, SZ, P, P]),
    "qg_index_free": (None, [P]),
    "qg_index_device_bytes": (SZ, [P]),
    "qg_search_batch": (C.c_int, [P, P, SZ, P, P, P, SZ, P, P, P, P]),
    "qg_search_batch_ex": (C.c_int, [P, P, SZ, P, P, P, SZ, P, P, P, P, SZ, P]),
    "qg_search_batch_noalloc": (C.c_int, [P, P, SZ, P, P, P, SZ, P, P, P, P]),
    "qg_search_noalloc_status": (C.c_int, [P]),
    "qg_search_batch_learned": (C.c_int, [P, P, SZ, P, P, P, SZ, P, P, P, P, P, P]),
    "qg_mlp_forward": (C.c_int, [P, SZ, P, P, P, P]),
    "qg_mlp_backward": (C.c_int, [P, P, SZ, P, P, P, P, P]),
    "qg_mlp_backward_mse": (C.c_int, [P, P, SZ, P, P, P, P, P]),
    "qg_mlp_adam": (C.c_int, [P, P, P, P, P, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, P]),
    "qg_index_set_launch": (C.c_int, [P, C.c_int, C.c_int]),
    "qg_index_set_tile": (C.c_int, [P, C.c_int]),
    "qg_index_max_block_warps": (C.c_int, [P]),
    "qg_index_share": (C.c_int, [P, C.POINTER(C.c_void_p)]),
    "qg_index_reserve": (C.c_int, [P, SZ, C.c_int, C.c_int]),
    "qg_search_batch_graph": (C.c_int, [P, P, SZ, P, P, P, P, SZ, P, P, P, P, P]),
    "qg_search_status": (C.c_int, [P, P]),
    "qg_center_mean": (C.c_int, [P, SZ, SZ, P, SZ, P, P]),
    "qg_encode_batch": (C.c_int, [P, P, SZ, P, P, P]),
    "qg_rotate_gemm": (C.c_int, [P, P, SZ, P, P, P]),
    "qg_encode_batch_gemm": (C.c_int, [P, P, SZ, P, P, P]),
    "qg_rotate_gemm_planes": (C.c_int, [P, P, SZ, P, P]),
    "qg_export_sidecar_device": (C.c_int, [P, P, SZ, SZ, P, P, P]),
    "qg_space_signs": (C.c_bool, [P, P]),
    "qg_space_set_signs": (C.c_bool, [P, P]),
    "qg_build_vamana_device": (C.c_int, [P, P, SZ, SZ, SZ, SZ, C.c_float, SZ, SZ, SZ, SZ, SZ, P, P, SZ, P, P]),
    "qg_prune_candidates": (C.c_int, [P, P, SZ, SZ, P, SZ, SZ, C.c_float, P, P, SZ, P]),
    "qg_prepare_batch": (C.c_int, [P, P, SZ, P, P, P, P, P]),
    "qg_dither_floor_pairs": (C.c_int, [P, P, P, SZ, P, P, P]),
    "qg_round_quotient_pairs": (C.c_int, [P, P, SZ, P, P, P]),
    "qg_gate_pairs": (C.c_int, [P, P, P, P, P, P, SZ, P, SZ, P, SZ, C.c_float, P, P]),
    "qg_gate_full_pairs": (C.c_int, [P, P, P, P, P, SZ, P, SZ, P, SZ, C.c_float, P, P]),
    "qg_distance_pairs": (C.c_int, [P, P, P, P, P, P, P, P, SZ, P, SZ, P, P, P]),
    "qg_residual_pairs": (C.c_int, [P, P, P, P, P, SZ, P, SZ, P, P, P]),
}

_lib = None


def exported_symbols() -> list[str]:
    """Names this module binds (every entry point of include/qgraph_gb300.h)."""
    return list(_SIGS)


def load(path: str | None = None):
    """Load the library (building it first if it is absent) and declare the signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def last_error() -> str:
    return (load().qg_last_error() or b"").decode(errors="replace")


def check(status: int, what: str) -> None:
    if status != QG_OK:
        raise RuntimeError(f"{what} failed: {STATUS_NAMES.get(status, status)}: {last_error()}")
