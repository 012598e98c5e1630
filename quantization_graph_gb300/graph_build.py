"""GPU graph construction.

build_vamana() is the reference's own build (rabitq_build_vamana_graph, rabitq_bridge.cpp:224-303:
bulk insertion in batches, refinement passes, grouped back-edges, robust_prune_4bit over the
symmetric 4-bit estimator) run on the GPU; it yields the reference's graph for the same
arguments (the reference spends 3202 s at 64 threads on it for 1M x 960).

build_graph() is this library's own faster builder, which does not reproduce the reference's
graph. Steps:

  1. exact-ish kNN candidates from the float vectors (TF32 GEMM through torch/cuBLAS, top-K),
     plus a few seeded random nodes per row (long-range candidates: on clustered data they are
     what the prune keeps as links between clusters, as Vamana's random initial graph does),
  2. alpha robust prune of the candidates to R out-edges on the GPU (qg_prune_candidates,
     symmetric 4-bit distances, occlusion with alpha 1.0 then alpha),
  3. reverse edges added as candidates and a second prune,
  4. optional refinement rounds: every node is searched with the batched beam search and the
     visited pool is pruned together with the current neighbours (the Vamana pass).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _native as N
from .space import RabitqSpace, _cuda, _ptr, _stream

NONE = -1  # UINT32_MAX viewed as int32


def knn_candidates(data: torch.Tensor, k: int, chunk: int = 4096) -> torch.Tensor:
    """[n, k] int32 nearest-neighbour ids (self excluded) by squared L2 (TF32 GEMM)."""
    n = data.shape[0]
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        norms = (data * data).sum(1)
        out = torch.empty((n, k), dtype=torch.int32, device=data.device)
        for s in range(0, n, chunk):
            e = min(n, s + chunk)
            d = torch.addmm(norms[None, :], data[s:e], data.T, beta=1.0, alpha=-2.0)
            d += norms[s:e, None]
            d[torch.arange(e - s, device=data.device), torch.arange(s, e, device=data.device)] = float("inf")
            out[s:e] = torch.topk(d, k, dim=1, largest=False, sorted=True).indices.to(torch.int32)
            del d
        return out
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def build_vamana(space: RabitqSpace, compact: torch.Tensor, r: int = 64, l_build: int = 400, alpha: float = 1.2,
                 beam: int = 1, batch: int = 4096, refine: int = 1, cap: int = 256, stop_hops: int = 2,
                 edge_stride: int | None = None) -> tuple[torch.Tensor, torch.Tensor, int]:
    """rabitq_build_vamana_graph over device compact records [n, compact_bytes] (uint8).
    Defaults are the formal run's (max degree 64, build beam 400, alpha 1.2, build beam width 1,
    batch 4096, refine 1, prune cap 256, early stop 2). Returns (degrees int32 [n], edges int32
    [n, edge_stride], zero past each degree, distances evaluated)."""
    lib = N.load()
    compact = _cuda(compact, torch.uint8)
    n = compact.shape[0]
    edge_stride = edge_stride or r
    deg = torch.empty(n, dtype=torch.int32, device="cuda")
    edges = torch.empty((n, edge_stride), dtype=torch.int32, device="cuda")
    evals = C.c_uint64(0)
    N.check(lib.qg_build_vamana_device(space.ptr, _ptr(compact), n, compact.shape[1], r, l_build, alpha, beam, batch,
                                       refine, cap, stop_hops, _ptr(deg), _ptr(edges), edge_stride,
                                       C.byref(evals), _stream()), "qg_build_vamana_device")
    return deg, edges, int(evals.value)


def prune(space: RabitqSpace, compact: torch.Tensor, candidates: torch.Tensor, r: int, alpha: float,
          edge_stride: int | None = None) -> tuple[torch.Tensor, torch.Tensor]:
    lib = N.load()
    n, k = candidates.shape
    edge_stride = edge_stride or r
    cand = _cuda(candidates, torch.int32)
    deg = torch.empty(n, dtype=torch.int32, device="cuda")
    edges = torch.empty((n, edge_stride), dtype=torch.int32, device="cuda")
    N.check(lib.qg_prune_candidates(space.ptr, _ptr(compact), compact.shape[1], n, _ptr(cand), k, r, alpha,
                                    _ptr(deg), _ptr(edges), edge_stride, _stream()), "qg_prune_candidates")
    return deg, edges


def reverse_candidates(edges: torch.Tensor, per_node: int) -> torch.Tensor:
    """[n, per_node] reverse neighbours (sources of in-edges), NONE padded."""
    n, r = edges.shape
    valid = edges.flatten() != NONE
    src = torch.arange(n, device=edges.device, dtype=torch.int64).repeat_interleave(r)[valid]
    dst = edges.flatten()[valid].to(torch.int64)
    order = torch.argsort(dst, stable=True)
    dst, src = dst[order], src[order]
    counts = torch.bincount(dst, minlength=n)
    starts = torch.cumsum(counts, 0) - counts
    rank = torch.arange(dst.numel(), device=edges.device) - starts[dst]
    keep = rank < per_node
    out = torch.full((n, per_node), NONE, dtype=torch.int32, device=edges.device)
    out[dst[keep], rank[keep]] = src[keep].to(torch.int32)
    return out


def reachable_fraction(edges: torch.Tensor, start: int = 0, max_rounds: int = 10_000) -> float:
    """Fraction of nodes reachable from `start` (breadth-first on the GPU)."""
    n = edges.shape[0]
    seen = torch.zeros(n, dtype=torch.bool, device=edges.device)
    seen[start] = True
    frontier = torch.tensor([start], device=edges.device, dtype=torch.int64)
    for _ in range(max_rounds):
        nb = edges[frontier].flatten()
        nb = nb[nb != NONE].to(torch.int64)
        nb = nb[~seen[nb]]
        if nb.numel() == 0:
            break
        nb = torch.unique(nb)
        seen[nb] = True
        frontier = nb
    return float(seen.float().mean())


def build_graph(space: RabitqSpace, data: torch.Tensor, compact: torch.Tensor, r: int = 64,
                knn: int = 128, alpha: float = 1.2, reverse: int = 64, refine_rounds: int = 0,
                refine_l: int = 128, residual=None, msb=None, factors=None,
                log=None, random_candidates: int = 16, seed: int = 0) -> tuple[torch.Tensor, torch.Tensor]:
    """Returns (degrees [n] int32, edges [n, r] int32 with -1 padding) on the GPU.

    refine_rounds > 0 needs residual/msb/factors: each round searches every node from node 0
    with list size refine_l, prunes the expanded nodes together with the current neighbours
    (the Vamana pass, vamana_index.h:452-528) and adds reverse edges."""
    from .index import OursIndex

    data = _cuda(data, torch.float32)
    n = data.shape[0]
    cand = knn_candidates(data, knn)
    if random_candidates > 0:
        g = torch.Generator(device=data.device)
        g.manual_seed(seed)
        rnd = torch.randint(0, n, (n, random_candidates), generator=g, device=data.device, dtype=torch.int32)
        cand = torch.cat([cand, rnd], dim=1)
    deg, edges = prune(space, compact, cand, r, alpha)
    del cand
    rev = reverse_candidates(edges, reverse)
    deg, edges = prune(space, compact, torch.cat([edges, rev], dim=1), r, alpha)
    del rev
    cap = 256 - r
    for rnd in range(refine_rounds):
        ix = OursIndex(space, compact, residual, msb, factors, deg, edges)
        chunks = [ix.search_expanded(data[s:s + 131072], l_value=refine_l, cap=cap)
                  for s in range(0, n, 131072)]
        expanded = torch.cat(chunks)
        del ix, chunks
        deg, edges = prune(space, compact, torch.cat([edges, expanded], dim=1), r, alpha)
        del expanded
        rev = reverse_candidates(edges, reverse)
        deg, edges = prune(space, compact, torch.cat([edges, rev], dim=1), r, alpha)
        if log:
            log(f"  graph refine round {rnd + 1} done")
    return deg, edges
