"""Serving uneven query batches with one captured CUDA graph, and the launch-shape autotuner.

GraphSearcher captures qg_search_batch_graph once (query preparation + the persistent search
kernel, plus the two counter resets) for the largest batch; every later batch -- any size up to
the maximum, any mix of per-query k and L -- only copies its queries, k, L and batch size into
the captured buffers and replays the graph. The kernels read the batch size on the device, so
nothing is re-captured and nothing is allocated per batch.

SearchPool keeps several batches in flight over one resident index (a searcher per handle from
OursIndex.share, a stream each), so small batches share the GPU instead of queueing.

autotune() times the persistent kernel's launch shapes (warps per block, resident blocks per
SM) and, for code dims of 1024 and more, the tile shapes of its gate and traversal loops
(qg_index_set_tile) on a sample of the workload and keeps the fastest on the index. Every shape
returns the same results; only the speed differs.
"""
from __future__ import annotations

import ctypes as C
import time

import torch

from . import _native as N
from .space import _cuda, _ptr


def autotune(index, queries: torch.Tensor, k: int, l_value: int, shapes=None, tiles=None, repeats: int = 3,
             log=None):
    """Pick (tile, warps_per_block, blocks_per_sm) for this index and pool size; returns the timings.

    The tile shapes (where the code dim is at least 1024, where they exist) are timed with the
    automatic launch shape, then the launch shapes with the best tile (its block width from
    qg_index_max_block_warps)."""
    lib = N.load()
    if tiles is None:
        tiles = [0, 1, 2, 3, 4] if index.space.code_dim >= 1024 else [0]
    q = _cuda(queries, torch.float32)
    ids = torch.empty((q.shape[0], k), dtype=torch.int32, device="cuda")
    dists = torch.empty((q.shape[0], k), dtype=torch.float32, device="cuda")

    def timed(wpb, per_sm, tile):
        N.check(lib.qg_index_set_tile(index.handle, tile), "qg_index_set_tile")
        N.check(lib.qg_index_set_launch(index.handle, wpb, per_sm), "qg_index_set_launch")
        index.search_into(q, ids, dists, k=k, l_value=l_value)
        torch.cuda.synchronize()
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(repeats):
            index.search_into(q, ids, dists, k=k, l_value=l_value)
        end.record()
        torch.cuda.synchronize()
        ms = start.elapsed_time(end) / repeats
        if log:
            log(f"  tile {tile}, launch {wpb or 'auto'} warps/block, <= {per_sm or 'max'} blocks/SM: {ms:.3f} ms")
        return ms

    results = [((0, 0, t), timed(0, 0, t)) for t in tiles]
    tile = min(results, key=lambda r: r[1])[0][2]
    N.check(lib.qg_index_set_tile(index.handle, tile), "qg_index_set_tile")
    w = lib.qg_index_max_block_warps(index.handle)
    shapes = shapes or [(w, 0), (max(1, w // 2), 0), (w, 1), (w, 2), (max(1, w // 2), 2)]
    results += [((wpb, per_sm, tile), timed(wpb, per_sm, tile)) for wpb, per_sm in shapes]
    best = min(results, key=lambda r: r[1])[0]
    N.check(lib.qg_index_set_tile(index.handle, best[2]), "qg_index_set_tile")
    N.check(lib.qg_index_set_launch(index.handle, best[0], best[1]), "qg_index_set_launch")
    return best, results


class GraphSearcher:
    def __init__(self, index, dim: int, max_batch: int, max_k: int, max_l: int, model=None,
                 threshold: float | None = None, rerank: int = 100):
        self.lib = N.load()
        self.index = index
        self.max_batch, self.max_k, self.max_l = max_batch, max_k, max_l
        N.check(self.lib.qg_index_reserve(index.handle, max_batch, max_l, max_k), "qg_index_reserve")
        self.q = torch.zeros((max_batch, dim), dtype=torch.float32, device="cuda")
        self.k = torch.full((max_batch,), max_k, dtype=torch.int32, device="cuda")
        self.l = torch.full((max_batch,), max_l, dtype=torch.int32, device="cuda")
        self.nq = torch.zeros(1, dtype=torch.int32, device="cuda")
        self.ids = torch.empty((max_batch, max_k), dtype=torch.int32, device="cuda")
        self.dists = torch.empty((max_batch, max_k), dtype=torch.float32, device="cuda")
        self.params = N.SearchParams(max_k, max_l, 1, 1.9, rerank, 0, 0)
        self.model = model.struct(threshold) if model is not None else None
        self.stream = torch.cuda.Stream()
        self.graph = torch.cuda.CUDAGraph()
        # one uncaptured call settles every lazy set-up, then the capture
        with torch.cuda.stream(self.stream):
            self.nq.fill_(1)
            self._launch()
        torch.cuda.synchronize()
        with torch.cuda.graph(self.graph, stream=self.stream):
            self._launch()
        torch.cuda.synchronize()

    def _launch(self):
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        model = C.byref(self.model) if self.model is not None else None
        N.check(self.lib.qg_search_batch_graph(self.index.handle, _ptr(self.q), self.max_batch, _ptr(self.nq),
                                               C.byref(self.params), _ptr(self.k), _ptr(self.l), self.max_k,
                                               _ptr(self.ids), _ptr(self.dists), None, model, st),
                "qg_search_batch_graph")

    def search(self, queries: torch.Tensor, k: torch.Tensor, l_value: torch.Tensor):
        """Replay the graph for one batch; returns views of the result buffers (valid until the
        next call) after the batch completes on the searcher's stream."""
        n = queries.shape[0]
        if n > self.max_batch:
            raise ValueError("batch larger than the captured maximum")
        self.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.stream):
            self.q[:n].copy_(queries, non_blocking=True)
            self.k[:n].copy_(k, non_blocking=True)
            self.l[:n].copy_(l_value, non_blocking=True)
            self.nq.fill_(n)  # the size travels as a kernel argument: no host buffer to race on
            self.graph.replay()
        return self.ids[:n], self.dists[:n]

    def synchronize(self):
        self.stream.synchronize()


class SearchPool:
    """Several batches in flight over one resident index: `inflight` GraphSearchers, each on a
    handle of its own (OursIndex.share: the same payload, separate scratch) and a stream of its
    own, take the batches in turn. A searcher is reused only after its previous batch completes,
    so the results of a batch stay valid until `inflight` more batches have been submitted."""

    def __init__(self, index, dim: int, max_batch: int, max_k: int, max_l: int, inflight: int = 4, model=None,
                 threshold: float | None = None, rerank: int = 100):
        self.handles = [index] + [index.share() for _ in range(max(1, inflight) - 1)]
        self.searchers = [GraphSearcher(h, dim, max_batch, max_k, max_l, model=model, threshold=threshold,
                                        rerank=rerank) for h in self.handles]
        self.next = 0
        self.busy = [None] * len(self.searchers)  # per searcher: (start, end) events of its batch

    def run(self, batches, out_ids=None):
        """Serve (queries, k, L) batches (host or device tensors) in order with up to `inflight` in
        flight; out_ids (pinned host [sum of batch sizes x max_k], optional) receives the ids.
        Returns per-batch device latencies (ms, start of the batch's copies to the end of its
        result copy, on its stream) and the elapsed wall seconds."""
        lat = []
        t_all = time.perf_counter()
        row = 0
        for qb, kb, lb in batches:
            i = self.next
            self.next = (i + 1) % len(self.searchers)
            gs = self.searchers[i]
            if self.busy[i] is not None:
                s, e = self.busy[i]
                e.synchronize()
                lat.append(s.elapsed_time(e))
            n = qb.shape[0]
            if n > gs.max_batch:
                raise ValueError("batch larger than the captured maximum")
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(gs.stream):
                s.record()
                gs.q[:n].copy_(qb, non_blocking=True)  # from pinned host memory: one H2D copy each
                gs.k[:n].copy_(kb, non_blocking=True)
                gs.l[:n].copy_(lb, non_blocking=True)
                gs.nq.fill_(n)
                gs.graph.replay()
                if out_ids is not None:
                    out_ids[row:row + n].copy_(gs.ids[:n], non_blocking=True)
                e.record()
            self.busy[i] = (s, e)
            row += n
        for i, b in enumerate(self.busy):
            if b is not None:
                b[1].synchronize()
                lat.append(b[0].elapsed_time(b[1]))
                self.busy[i] = None
        return lat, time.perf_counter() - t_all


def serve(searcher: GraphSearcher, batches, log=None):
    """Run a list of (queries, k, L) batches back to back; returns per-batch latencies (ms, host
    wall clock from submission to completion) and the total elapsed seconds."""
    lat = []
    outs = []
    t_all = time.perf_counter()
    for qb, kb, lb in batches:
        t0 = time.perf_counter()
        ids, dists = searcher.search(qb, kb, lb)
        searcher.synchronize()
        lat.append((time.perf_counter() - t0) * 1000.0)
        outs.append(ids.clone())
    return lat, time.perf_counter() - t_all, outs
