"""Learned early termination for the batched search (no counterpart in the reference).

A network 8 -> 64 -> 64 -> 1 (BF16 weights, FP32 accumulation) reads the search state every
`every` hops inside the search kernel: hops / L, the spread of the current top-k, hops since
the top k last changed / L, hops since the first max(rerank, k) pool entries last changed / L,
unexpanded fraction, position and distance of the next expansion, log ||q - c||^2. Two ways to
use it:

  stop classifier (kind 0): stop when sigmoid(output) exceeds a threshold; a checkpoint is a
      positive example when the first max(rerank, k) pool entries already hold every id the
      full fixed-L search returns.
  hop budget (kind 1, after Li, Zhang, Andersen and He, "Improving Approximate Nearest Neighbor
      Search through Learned Adaptive Early Termination", SIGMOD 2020): the output regresses
      log(h*), h* being the hop at which the query's pool first holds every id of the full
      search's result; the query stops once its hops reach scale * exp(output). The scale is
      the one knob tuned against the recall target.

Plain fixed-L search stays the fallback and the judge: training targets come from it, and every
recall is measured against it. Training runs on the GPU with this library's own kernels
(qg_mlp_backward / qg_mlp_backward_mse, qg_mlp_adam).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from .space import _cuda, _ptr, _stream

IN, HIDDEN = 8, 64
PARAMS = N.MLP_PARAMS


def init_weights(seed: int = 0) -> torch.Tensor:
    """He-initialised FP32 master weights in the packed layout."""
    g = torch.Generator().manual_seed(seed)
    w = torch.zeros(PARAMS, dtype=torch.float32)
    o = 0
    w[o:o + HIDDEN * IN] = torch.randn(HIDDEN * IN, generator=g) * (2.0 / IN) ** 0.5
    o += HIDDEN * IN + HIDDEN
    w[o:o + HIDDEN * HIDDEN] = torch.randn(HIDDEN * HIDDEN, generator=g) * (2.0 / HIDDEN) ** 0.5
    o += HIDDEN * HIDDEN + HIDDEN
    w[o:o + HIDDEN] = torch.randn(HIDDEN, generator=g) * (1.0 / HIDDEN) ** 0.5
    return w.cuda()


def to_bf16_bits(w: torch.Tensor) -> torch.Tensor:
    """FP32 -> BF16 (round to nearest even) as raw uint16 bits in an int16 tensor."""
    return w.to(torch.bfloat16).view(torch.int16).contiguous()


KIND_CLASSIFIER, KIND_BUDGET = 0, 1


@dataclass
class StopModel:
    weights: torch.Tensor   # [PARAMS] int16 holding BF16 bits (device)
    norm: torch.Tensor      # [16] float32: mean[8], inv_std[8] (device)
    every: int = 4
    min_hops: int = 8
    kind: int = KIND_CLASSIFIER
    predict_once: bool = False

    def struct(self, knob: float) -> N.StopModel:
        """knob: the threshold of a classifier, the budget scale of a hop budget."""
        if self.kind == KIND_CLASSIFIER:
            return N.StopModel(self.weights.data_ptr(), self.norm.data_ptr(), float(knob), self.every,
                               self.min_hops, KIND_CLASSIFIER, 0.0, 0)
        return N.StopModel(self.weights.data_ptr(), self.norm.data_ptr(), 0.5, self.every, self.min_hops,
                           KIND_BUDGET, float(knob), 1 if self.predict_once else 0)


@dataclass
class Traces:
    features: torch.Tensor    # [rows, 8] search-state features at the checkpoints
    found: torch.Tensor       # [rows] truth ids already in the first max(rerank, k) pool entries
    query: torch.Tensor       # [rows] int64 query index of the row
    hop: torch.Tensor         # [rows] int64 hop count at the checkpoint
    final_hops: torch.Tensor  # [nq] int64 hops of the full search
    truth_k: int

    def classifier_labels(self) -> torch.Tensor:
        """1 where every truth id is already in the rerank window."""
        return (self.found >= self.truth_k).to(torch.float32)

    def hops_needed(self) -> torch.Tensor:
        """[nq] h*: the first checkpoint hop whose rerank window holds every truth id (the
        window only loses an id to closer entries, and the truth ids are the final result, so
        this is monotone), else the full search's hop count."""
        nq = self.final_hops.shape[0]
        big = torch.iinfo(torch.int64).max
        first = torch.full((nq,), big, dtype=torch.int64, device=self.hop.device)
        done = self.found >= self.truth_k
        first.scatter_reduce_(0, self.query[done], self.hop[done], reduce="amin")
        return torch.where(first == big, self.final_hops, torch.minimum(first, self.final_hops))

    def budget_targets(self) -> torch.Tensor:
        """log(h*) of each row's query: the hop-budget regression target."""
        h = self.hops_needed().clamp_min(1).to(torch.float32)
        return torch.log(h)[self.query]


def collect_traces(index, queries: torch.Tensor, truth: torch.Tensor, k: int, l_value: int, every: int = 4,
                   cap: int | None = None, rerank: int = 100) -> Traces:
    """Feature rows from a plain fixed-L search of `queries` (one row every `every` hops), each
    with the number of `truth` ids [nq, >=k] (the ids the full search returns) already in the
    rerank window."""
    lib = N.load()
    q = _cuda(queries, torch.float32)
    nq = q.shape[0]
    cap = cap or (4 * l_value) // every + 8
    tk = int(min(k, truth.shape[1]))
    tr = _cuda(truth[:, :tk], torch.int32)
    feat = torch.empty((nq, cap, IN), dtype=torch.float32, device="cuda")
    lab = torch.empty((nq, cap), dtype=torch.float32, device="cuda")
    cnt = torch.empty(nq, dtype=torch.int32, device="cuda")
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
    params = N.SearchParams(k, l_value, 1, 1.9, rerank, 0, 0)
    treq = N.TraceRequest(tr.data_ptr(), tk, every, cap, feat.data_ptr(), lab.data_ptr(), cnt.data_ptr())
    N.check(lib.qg_search_batch_learned(index.handle, _ptr(q), nq, C.byref(params), None, None, k, _ptr(ids),
                                        _ptr(dists), _ptr(stats), None, C.byref(treq), _stream()), "trace search")
    N.check(lib.qg_search_status(index.handle, _stream()), "trace search status")
    mask = torch.arange(cap, device="cuda")[None, :] < cnt[:, None]
    qidx = torch.arange(nq, device="cuda")[:, None].expand(nq, cap)
    hop = (torch.arange(cap, device="cuda")[None, :] + 1).expand(nq, cap) * every
    return Traces(feat[mask], lab[mask], qidx[mask], hop[mask], stats[:, 2].clone(), tk)


def forward(weights_bf16: torch.Tensor, norm: torch.Tensor, x: torch.Tensor) -> torch.Tensor:
    lib = N.load()
    x = _cuda(x, torch.float32)
    out = torch.empty(x.shape[0], dtype=torch.float32, device="cuda")
    N.check(lib.qg_mlp_forward(_ptr(x), x.shape[0], _ptr(norm), _ptr(weights_bf16), _ptr(out), _stream()),
            "qg_mlp_forward")
    return out


def loss_and_grad(weights_bf16: torch.Tensor, norm: torch.Tensor, x: torch.Tensor, y: torch.Tensor,
                  kind: int = KIND_CLASSIFIER):
    lib = N.load()
    x = _cuda(x, torch.float32)
    y = _cuda(y, torch.float32)
    grad = torch.empty(PARAMS, dtype=torch.float32, device="cuda")
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    backward = lib.qg_mlp_backward_mse if kind == KIND_BUDGET else lib.qg_mlp_backward
    N.check(backward(_ptr(x), _ptr(y), x.shape[0], _ptr(norm), _ptr(weights_bf16), _ptr(grad), _ptr(loss),
                     _stream()), "qg_mlp_backward")
    return loss, grad


def train(features: torch.Tensor, labels: torch.Tensor, epochs: int = 4, batch: int = 8192,
          lr: float = 2e-3, seed: int = 0, every: int = 4, min_hops: int = 8, log=None,
          kind: int = KIND_CLASSIFIER, predict_once: bool = False) -> StopModel:
    """Adam with the library's kernels on the BCE loss (a stop classifier, labels in {0, 1}) or
    on the squared error (a hop budget, labels = log of the hops needed); returns the BF16 model."""
    lib = N.load()
    x = _cuda(features, torch.float32)
    y = _cuda(labels, torch.float32)
    mean = x.mean(0)
    std = x.std(0).clamp_min(1e-6)
    norm = torch.cat([mean, 1.0 / std]).contiguous()
    master = init_weights(seed)
    if kind == KIND_BUDGET:
        master[PARAMS - 1] = y.mean()  # the output bias starts at the mean target
    backward = lib.qg_mlp_backward_mse if kind == KIND_BUDGET else lib.qg_mlp_backward
    w = to_bf16_bits(master)
    m = torch.zeros_like(master)
    v = torch.zeros_like(master)
    grad = torch.empty(PARAMS, dtype=torch.float32, device="cuda")
    loss = torch.empty(1, dtype=torch.float32, device="cuda")
    gen = torch.Generator(device="cuda").manual_seed(seed)
    step = 0
    n = x.shape[0]
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen, device="cuda")
        tot = 0.0
        for s in range(0, n, batch):
            idx = perm[s:s + batch]
            xb = x[idx].contiguous()
            yb = y[idx].contiguous()
            N.check(backward(_ptr(xb), _ptr(yb), xb.shape[0], _ptr(norm), _ptr(w), _ptr(grad), _ptr(loss),
                             _stream()), "qg_mlp_backward")
            step += 1
            N.check(lib.qg_mlp_adam(_ptr(master), _ptr(w), _ptr(grad), _ptr(m), _ptr(v), lr, 0.9, 0.999, 1e-8,
                                    step, _stream()), "qg_mlp_adam")
            tot += float(loss) * xb.shape[0]
        if log:
            what = "squared error / 2" if kind == KIND_BUDGET else "BCE"
            log(f"  stop-model epoch {ep + 1}: mean {what} {tot / n:.4f} over {n} rows")
    return StopModel(w, norm, every=every, min_hops=min_hops, kind=kind, predict_once=predict_once)


def search(index, queries: torch.Tensor, model: StopModel, threshold: float, k: int = 10, l_value: int = 100,
           rerank: int = 100, ids_out: torch.Tensor | None = None, dists_out: torch.Tensor | None = None,
           stats_out: torch.Tensor | None = None):
    """Batched search with the learned stop (stream-ordered; outputs preallocated or new).
    `threshold` is the classifier's threshold, or the budget scale of a hop-budget model."""
    lib = N.load()
    q = _cuda(queries, torch.float32)
    nq = q.shape[0]
    ids = ids_out if ids_out is not None else torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dists = dists_out if dists_out is not None else torch.empty((nq, k), dtype=torch.float32, device="cuda")
    params = N.SearchParams(k, l_value, 1, 1.9, rerank, 0, 0)
    sm = model.struct(threshold)
    N.check(lib.qg_search_batch_learned(index.handle, _ptr(q), nq, C.byref(params), None, None, ids.shape[1],
                                        _ptr(ids), _ptr(dists), _ptr(stats_out), C.byref(sm), None, _stream()),
            "learned-stop search")
    return ids, dists
