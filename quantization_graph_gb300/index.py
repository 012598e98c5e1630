"""Device-resident Ours-DiskANN index and its batched search: the host side of the path
that diskann_runner::run_ours_exrabitq4 drives (experiments/02_diskann_fair/src/
diskann_runner.rs:155-445): encode payloads, load a graph built by the reference (or build
one), export the paper-prune sidecar, then search a batch of queries with
search_ours_paper_active's knobs (ours_diskann.rs:1174-1227).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .space import RabitqSpace, _cuda, _ptr, _stream

STATS_DTYPE = np.dtype([(f, "<u8") for f in N.STATS_FIELDS])


@dataclass
class SearchResult:
    ids: torch.Tensor        # [nq, k] int64 view of uint32 ids (UINT32_MAX = none)
    distances: torch.Tensor  # [nq, k] float32 reranked estimates (+inf = none)
    stats: np.ndarray | None  # [nq] OursPaperSearchStats counters


class OursIndex:
    """Payloads + adjacency resident in HBM (structure-of-arrays, 16-byte aligned rows)."""

    def __init__(self, space: RabitqSpace, compact, residual, msb, factors, degrees, edges,
                 base_points: int | None = None, total_points: int | None = None):
        self.space = space
        self.lib = N.load()
        compact = _cuda(compact, torch.uint8)
        residual = _cuda(residual, torch.uint8)
        msb = _cuda(msb, torch.uint8)
        factors = _cuda(factors, torch.uint8)
        degrees = _cuda(torch.as_tensor(np.asarray(degrees, np.uint32).view(np.int32))
                        if isinstance(degrees, np.ndarray) else degrees, torch.int32)
        edges = _cuda(torch.as_tensor(np.asarray(edges, np.uint32).view(np.int32))
                      if isinstance(edges, np.ndarray) else edges, torch.int32)
        self.base_points = int(base_points if base_points is not None else compact.shape[0])
        self.total_points = int(total_points if total_points is not None else degrees.shape[0])
        self.max_degree = int(edges.shape[1])
        handle = C.c_void_p()
        N.check(self.lib.qg_index_upload_device(
            space.ptr, _ptr(compact), compact.shape[1], _ptr(residual), residual.shape[1], _ptr(msb),
            msb.shape[1], _ptr(factors), factors.shape[1], _ptr(degrees), _ptr(edges), edges.shape[1],
            self.base_points, self.total_points, _stream(), C.byref(handle)), "qg_index_upload_device")
        self.handle = handle

    def __del__(self):
        try:
            self.lib.qg_index_free(self.handle)
        except Exception:
            pass

    @classmethod
    def build_from_vectors(cls, space: RabitqSpace, data: torch.Tensor, degrees, edges,
                           total_points: int | None = None) -> "OursIndex":
        """Encode `data` on the GPU, export the sidecar, attach an adjacency (the path of
        run_ours_exrabitq4 with --graph-file: encode, copy_shared_graph, export sidecar)."""
        compact, residual = space.encode(data)
        msb, factors = space.export_paper_sidecar(compact)
        return cls(space, compact, residual, msb, factors, degrees, edges, base_points=data.shape[0],
                   total_points=total_points)

    def device_bytes(self) -> int:
        return self.lib.qg_index_device_bytes(self.handle)

    def share(self) -> "OursIndex":
        """A second handle on this index's resident payload (qg_index_share: no copy, its own
        search scratch), for searches that run at the same time on another stream."""
        other = object.__new__(OursIndex)
        other.space, other.lib = self.space, self.lib
        other.base_points, other.total_points, other.max_degree = self.base_points, self.total_points, self.max_degree
        other._source = self  # keeps the space and the first handle alive
        handle = C.c_void_p()
        N.check(self.lib.qg_index_share(self.handle, C.byref(handle)), "qg_index_share")
        other.handle = handle
        return other

    def search_into(self, queries: torch.Tensor, ids_out: torch.Tensor, dists_out: torch.Tensor,
                    k: int = 10, l_value: int = 100, beam_width: int = 1, epsilon0: float = 1.9,
                    rerank_candidates: int = 100, early_stop_hops: int = 0, kth_stop: bool = False,
                    stats_out: torch.Tensor | None = None, k_per_query: torch.Tensor | None = None,
                    l_per_query: torch.Tensor | None = None, fused_int_rerank: bool | None = None) -> None:
        """Stream-ordered search writing into preallocated CUDA outputs (no host sync).
        fused_int_rerank: rerank an Int8 / Int4 traversal with the fused restore + residual
        kernel's arithmetic; None reads RABITQ_ENABLE_FUSED_INT_RERANK as the reference does
        (ours_diskann.rs:1166-1172)."""
        if fused_int_rerank is None:
            fused_int_rerank = os.environ.get("RABITQ_ENABLE_FUSED_INT_RERANK") is not None
        params = N.SearchParams(k, l_value, beam_width, epsilon0, rerank_candidates, early_stop_hops,
                                1 if kth_stop else 0, 1 if fused_int_rerank else 0)
        N.check(self.lib.qg_search_batch(self.handle, _ptr(queries), queries.shape[0], C.byref(params),
                                         _ptr(k_per_query), _ptr(l_per_query), ids_out.shape[1], _ptr(ids_out),
                                         _ptr(dists_out), _ptr(stats_out), _stream()), "qg_search_batch")

    def search_expanded(self, queries, l_value: int, cap: int, k: int = 1) -> torch.Tensor:
        """[nq, cap] int32 ids of the nodes each query expanded, in hop order (-1 padding)."""
        q = _cuda(queries, torch.float32)
        nq = q.shape[0]
        ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
        dists = torch.empty((nq, k), dtype=torch.float32, device="cuda")
        expanded = torch.empty((nq, cap), dtype=torch.int32, device="cuda")
        params = N.SearchParams(k, l_value, 1, 1.9, 0, 0, 0)
        N.check(self.lib.qg_search_batch_ex(self.handle, _ptr(q), nq, C.byref(params), None, None, k, _ptr(ids),
                                            _ptr(dists), None, _ptr(expanded), cap, _stream()), "qg_search_batch_ex")
        return expanded

    def search(self, queries, k: int = 10, l_value: int = 100, beam_width: int = 1,
               epsilon0: float = 1.9, rerank_candidates: int = 100, early_stop_hops: int = 0,
               kth_stop: bool = False, with_stats: bool = True, k_per_query=None,
               l_per_query=None, fused_int_rerank: bool | None = None) -> SearchResult:
        """Batched search_ours_paper_active with the space's query codec; checks the device status."""
        q = _cuda(queries, torch.float32)
        nq = q.shape[0]
        kmax = int(max(k, int(torch.as_tensor(k_per_query).max())) if k_per_query is not None else k)
        lmax = int(max(l_value, int(torch.as_tensor(l_per_query).max())) if l_per_query is not None else l_value)
        kq = _cuda(k_per_query, torch.int32) if k_per_query is not None else None
        lq = _cuda(l_per_query, torch.int32) if l_per_query is not None else None
        ids = torch.empty((nq, kmax), dtype=torch.int32, device="cuda")
        dists = torch.empty((nq, kmax), dtype=torch.float32, device="cuda")
        stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda") if with_stats else None
        self.search_into(q, ids, dists, k=kmax, l_value=lmax, beam_width=beam_width, epsilon0=epsilon0,
                         rerank_candidates=rerank_candidates, early_stop_hops=early_stop_hops,
                         kth_stop=kth_stop, stats_out=stats, k_per_query=kq, l_per_query=lq,
                         fused_int_rerank=fused_int_rerank)
        N.check(self.lib.qg_search_status(self.handle, _stream()), "search status")
        st = None
        if stats is not None:
            st = stats.cpu().numpy().view(STATS_DTYPE).reshape(nq)
        return SearchResult(ids.to(torch.int64) & 0xFFFFFFFF, dists, st)
