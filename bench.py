#!/usr/bin/env python
"""Benchmark: QPS at recall@10 >= 0.95 of the Ours-DiskANN query path on one GB300.

Workload (default): 1,000,000 base vectors x 1536-d, unit-norm anisotropic Gaussian
(lambda_i ~ i^-0.8, seeded rotation), 10,000 queries drawn the same way, ExRaBitQ4 block16
encoding on the GPU, degree-64 graph built by the reference's Vamana algorithm on the GPU
(rabitq_build_vamana_graph with the formal arguments: L_build 400, alpha 1.2, batch 4096, refine
1, prune cap 256, early stop 2; the same graph the reference builds; --graph own selects this
library's faster kNN + prune builder), k = 10, INT8 query codec with the 1-bit paper-prune gate,
residual4 top-100 rerank, fixed-L beam search with the smallest L from a sweep that reaches
recall@10 >= 0.95 against an exact, certified FP64 ground truth.

One step = one batched search of all queries (one qg_search_batch: query preparation +
persistent search kernel). `value` is device-timed with inputs resident in HBM; `e2e` adds the
pinned host->device copy of the queries and the device->host copy of ids and distances.
The index (~2.6 GB) exceeds the 129 MB L2, so no flush is needed between steps.

Checks made on the run that is reported (`parity`, `encode_parity`, `ground_truth`): the
reference search restated on the CPU (oracle/) is run over a sample of the same queries at the
same L and must give the same ids, distance bits and the 9 counters as the GPU (the bench exits
non-zero otherwise); a seeded sample of the base is re-encoded by the oracle encoder and compared
with the GPU records byte for byte.

--impl reference times the reference's search on the host cores instead (the oracle's CPU
restatement, all threads) on the same index, queries and L: a set-up process builds the index on
the GPU and writes it to a temporary cache; the timed process reads the cache and loads only the
oracle. Each step is a bounded slice of the queries.
Multi-GPU (torchrun): query-sharded replicas -- every rank holds the whole index and searches the
queries of its id range; value counts each query once, at the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "QPS@recall10=0.95, 1M×1536 4-bit, learned-stop vs fixed-L beam, 1 GB300"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000)
    ap.add_argument("--dim", type=int, default=1536)
    ap.add_argument("--nq", type=int, default=10_000)
    ap.add_argument("--M", type=int, default=64)
    ap.add_argument("--k", type=int, default=10)
    ap.add_argument("--target-recall", type=float, default=0.95)
    ap.add_argument("--L", type=int, default=0, help="fixed L (0 = sweep)")
    ap.add_argument("--tile", type=int, default=-1, help="search tile shape (qg_index_set_tile: -1 by index size, 0..4)")
    ap.add_argument("--launch", default="", help="warps per block and blocks per SM, e.g. 7,3 (qg_index_set_launch)")
    ap.add_argument("--inflight", type=int, default=2,
                    help="timed steps in flight: step s runs on handle s mod N (qg_index_share: the same resident "
                         "index, search scratch of its own) and a stream of its own, so the next batch takes the "
                         "SMs the last queries of the previous one leave idle; 1 = one step after another")
    ap.add_argument("--codecs", default="int4,b1,b1main,full,int8_fused",
                    help="query codecs measured beside the Int8 headline on the same index (empty: none)")
    ap.add_argument("--codec-parity-queries", type=int, default=200)
    ap.add_argument("--parity-queries", type=int, default=1000,
                    help="queries re-run by the CPU restatement at the headline L and compared bit for bit")
    ap.add_argument("--encode-parity-rows", type=int, default=10_000,
                    help="base rows re-encoded by the oracle encoder and compared with the GPU records")
    ap.add_argument("--ref-step-seconds", type=float, default=0.5,
                    help="--impl reference: host time of one step (a slice of queries, one per thread)")
    ap.add_argument("--skip-cpu", action="store_true", help="no CPU parity leg (and no cpu_baseline)")
    ap.add_argument("--graph", default="reference", choices=["reference", "own"],
                    help="reference: the reference's Vamana build (rabitq_build_vamana_graph) on the GPU with the "
                         "formal arguments; own: this library's kNN + prune builder")
    ap.add_argument("--l-build", type=int, default=400, help="build search list size (--graph reference)")
    ap.add_argument("--refine", type=int, default=1, help="graph refinement rounds")
    ap.add_argument("--knn", type=int, default=240, help="kNN candidates per node for the graph")
    ap.add_argument("--refine-l", type=int, default=256, help="search list size of the refinement rounds")
    ap.add_argument("--no-learned", action="store_true", help="fixed-L only")
    ap.add_argument("--train-queries", type=int, default=50_000)
    ap.add_argument("--stop-every", type=int, default=8)
    ap.add_argument("--stop-epochs", type=int, default=4)
    ap.add_argument("--stop-kind", default="both", choices=["classifier", "budget", "both"],
                    help="learned stop: a stop classifier, a hop budget (LAET-style), or both (the faster wins)")
    ap.add_argument("--workload", default="dbpedia1536", choices=["dbpedia1536", "gist960", "stream", "encode"],
                    help="gist960: 1M x 960 |x| with lambda_i ~ i^-1.2; stream: uneven batched stream over "
                         "a 120k x 1024 clustered index; encode: the GPU encode with the rotation on the tensor "
                         "cores against the reference encoder")
    ap.add_argument("--stream-n", type=int, default=120_000)
    ap.add_argument("--stream-queries", type=int, default=200_000)
    ap.add_argument("--stream-inflight", type=int, default=8, help="batches in flight (SearchPool)")
    ap.add_argument("--stream-thresholds", default="0.9,0.95,0.98",
                    help="learned-stop thresholds tried on the stream ('' = fixed per-query L only)")
    ap.add_argument("--setup-cache", default="", help=argparse.SUPPRESS)  # internal: the reference arm's set-up
    args = ap.parse_args(argv)
    if args.workload == "gist960" and args.dim == 1536:
        args.dim = 960
    return args


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def fp32_score_error_bound(dim: int, base_norm_max: float, query_norm):
    """Bound on |e - (|b|^2 - 2 q.b)| for the FP32 shortlist score e = fl(|b|^2) - 2 fl(q.b):
    each FP32 sum or dot product of n terms, in any order, errs by at most gamma_n times the sum
    of the magnitudes (Higham 2002, section 3.1), gamma_n = n u / (1 - n u), u = 2^-24, plus one
    rounding of the final combination; |q.b| <= |q| |b| bounds the dot product's magnitudes."""
    u = 2.0 ** -24
    n = dim + 2
    gamma = n * u / (1.0 - n * u)
    b = base_norm_max
    return 1.01 * gamma * (b * b + 2.0 * query_norm * b)


def ground_truth(torch, base, queries, k, shortlist=64):
    """Exact top-k under FP64 distances, certified per query. An FP32 GEMM scores every base row
    (|b|^2 - 2 q.b, TF32 off) and keeps the `shortlist` best; these are re-scored in FP64. A query
    is certified when its k-th FP64 score lies below the shortlist's worst FP32 score minus the
    FP32 error bound: then no row outside the shortlist can enter the top k. Queries that fail
    the test are re-scored against the whole base in FP64. Returns (ids [nq, k], info)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        bn = (base * base).sum(1)
        bmax = float(bn.max().sqrt()) * (1.0 + 1e-6)
        nq = queries.shape[0]
        out = torch.empty((nq, k), dtype=torch.int64, device=base.device)
        failed = []
        for s in range(0, nq, 1024):
            q = queries[s:s + 1024]
            d = torch.addmm(bn[None, :], q, base.T, beta=1.0, alpha=-2.0)
            top = torch.topk(d, shortlist, dim=1, largest=False)
            del d
            cand = top.indices
            worst = top.values.max(dim=1).values.double()
            qd = q.double()
            diff = base[cand].double() - qd[:, None, :]
            dd = (diff * diff).sum(-1)                       # exact |q - b|^2 in FP64
            order = torch.argsort(dd, dim=1, stable=True)[:, :k]
            out[s:s + q.shape[0]] = torch.gather(cand, 1, order)
            kth = torch.gather(dd, 1, order[:, k - 1:k]).squeeze(1) - (qd * qd).sum(1)  # |b|^2 - 2 q.b
            qn = q.norm(dim=1).double()
            bound = torch.tensor([fp32_score_error_bound(base.shape[1], bmax, float(x)) for x in qn.tolist()],
                                 dtype=torch.float64, device=base.device)
            ok = kth + 1e-9 * (1.0 + kth.abs()) < worst - bound
            failed.extend((s + torch.nonzero(~ok).squeeze(1)).tolist())
        if failed:
            fq = queries[failed].double()
            best_d = torch.full((len(failed), k), float("inf"), dtype=torch.float64, device=base.device)
            best_i = torch.zeros((len(failed), k), dtype=torch.int64, device=base.device)
            for c in range(0, base.shape[0], 65536):
                bc = base[c:c + 65536].double()
                d = (bc * bc).sum(1)[None, :] - 2.0 * fq @ bc.T + (fq * fq).sum(1)[:, None]
                ids = torch.arange(c, c + bc.shape[0], device=base.device)[None, :].expand(len(failed), -1)
                alld = torch.cat([best_d, d], 1)
                alli = torch.cat([best_i, ids], 1)
                order = torch.argsort(alld, dim=1, stable=True)[:, :k]
                best_d = torch.gather(alld, 1, order)
                best_i = torch.gather(alli, 1, order)
            out[failed] = best_i
        info = {"method": f"FP32 GEMM shortlist of {shortlist} re-scored in FP64, certified per query by the FP32 "
                          "error bound; uncertified queries re-scored against the whole base in FP64",
                "queries": nq, "certified": nq - len(failed), "full_fp64_scan": len(failed)}
        return out, info
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def recall_at(ids, gt, k):
    hit = (ids[:, :k, None] == gt[:, None, :k]).any(-1).sum().item()
    return hit / (ids.shape[0] * k)


def recall_np(ids, gt, k):
    ids = np.asarray(ids, np.int64)[:, :k]
    gt = np.asarray(gt, np.int64)[:, :k]
    return float((ids[:, :, None] == gt[:, None, :]).any(-1).sum() / (ids.shape[0] * k))


def graph_desc(args) -> str:
    if args.graph == "reference":
        return (f"the reference's Vamana build (rabitq_build_vamana_graph) on the GPU, identical graph: R={args.M}, "
                f"L_build={args.l_build}, alpha 1.2, beam 1, batch 4096, refine {args.refine}, prune cap 256, "
                f"early stop 2")
    return (f"GPU kNN-{args.knn or 2 * args.M} + 16 random + alpha-1.2 prune + reverse edges + "
            f"{args.refine} search-based refinement round(s) at L={args.refine_l}")


def workload_config(args) -> dict:
    """The workload both arms run (identical in their JSON lines): data, index and search knobs."""
    metric = METRIC
    if (args.n, args.dim) != (1_000_000, 1536):  # another size: the metric names it
        size = f"{args.n // 1_000_000}M" if args.n % 1_000_000 == 0 else (
            f"{args.n // 1000}k" if args.n % 1000 == 0 else str(args.n))
        metric = METRIC.replace("1M×1536", f"{size}×{args.dim}")
    data_desc = f"{args.n} x {args.dim} unit-norm anisotropic (lambda_i ~ i^-0.8)"
    if args.workload == "gist960":
        metric = "QPS@recall10=0.95, 1M×960 4-bit, fixed-L beam, 1 GB300"
        data_desc = f"{args.n} x {args.dim} |x|, x ~ N(0, Q diag(i^-1.2) Q^T)"
    config = {"workload": (f"{data_desc}, M={args.M}, {args.nq} queries, k={args.k}, INT8 paper-prune gate, "
                           "residual4 rerank 100"),
              "n": args.n, "dim": args.dim, "queries": args.nq, "M": args.M, "k": args.k,
              "graph": graph_desc(args), "recall_target": args.target_recall,
              "operating_point": "smallest fixed L reaching the recall target (coarse sweep, then steps of 16)",
              "l2": "index larger than L2 (no flush needed)"}
    return metric, config


def build_workload(torch, args, log):
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.graph_build import build_graph, build_vamana, reachable_fraction
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace, train_global_center

    t0 = time.time()
    if args.workload == "gist960":  # |x|, x ~ N(0, Q diag(i^-1.2) Q^T)
        base = synthetic.anisotropic_torch(args.n, args.dim, 1.2, seed=1, absolute=True)
        queries = synthetic.anisotropic_torch(args.nq, args.dim, 1.2, seed=2, absolute=True)
    else:
        base = synthetic.anisotropic_torch(args.n, args.dim, 0.8, seed=1, normalize=True)
        queries = synthetic.anisotropic_torch(args.nq, args.dim, 0.8, seed=2, normalize=True)
    center = train_global_center(base)
    space = RabitqSpace(args.dim, center)
    torch.cuda.synchronize()
    t1 = time.time()
    compact, residual = space.encode(base)
    torch.cuda.synchronize()
    t_encode = time.time() - t1
    msb, factors = space.export_paper_sidecar(compact)
    t2 = time.time()
    if args.graph == "reference":  # max degree M, build beam 400, alpha 1.2, beam 1, batch 4096, refine 1,
        # prune cap 256, early stop 2 (scripts/local_runs/build_agnews_dbpedia_prereqs.sh, diskann_runner.rs:286-296)
        deg, edges, _ = build_vamana(space, compact, r=args.M, l_build=args.l_build, alpha=1.2, beam=1, batch=4096,
                                     refine=args.refine, cap=256, stop_hops=2)
    else:
        deg, edges = build_graph(space, base, compact, r=args.M, knn=args.knn or 2 * args.M, alpha=1.2,
                                 reverse=args.M, refine_rounds=args.refine, refine_l=args.refine_l, residual=residual,
                                 msb=msb, factors=factors)
    torch.cuda.synchronize()
    t_graph = time.time() - t2
    reach = reachable_fraction(edges)
    t3 = time.time()
    gt, gt_info = ground_truth(torch, base, queries, args.k)
    gt_info["seconds"] = round(time.time() - t3, 2)
    index = OursIndex(space, compact, residual, msb, factors, deg, edges)
    if args.tile != -1 or args.launch:
        from quantization_graph_gb300 import _native as N
        N.check(N.load().qg_index_set_tile(index.handle, args.tile), "qg_index_set_tile")
        if args.launch:
            wpb, per_sm = (int(x) for x in args.launch.split(","))
            N.check(N.load().qg_index_set_launch(index.handle, wpb, per_sm), "qg_index_set_launch")
    torch.cuda.empty_cache()
    log(f"setup: data {t1 - t0:.1f}s encode {t_encode:.2f}s graph {t_graph:.1f}s reachable {reach:.4f} "
        f"index {index.device_bytes() / 1e9:.2f} GB; ground truth {gt_info['certified']} certified, "
        f"{gt_info['full_fp64_scan']} by full FP64 scan")
    return dict(base=base, queries=queries, space=space, index=index, gt=gt, gt_info=gt_info, compact=compact,
                residual=residual, msb=msb, factors=factors, deg=deg, edges=edges, t_encode=t_encode,
                t_graph=t_graph, reach=reach)


def pick_l(torch, w, args, log):
    if args.L:
        r = w["index"].search(w["queries"], k=args.k, l_value=args.L, with_stats=False)
        return args.L, recall_at(r.ids, w["gt"], args.k), {args.L: recall_at(r.ids, w["gt"], args.k)}
    sweep = {}
    chosen = None
    for L in (10, 16, 24, 32, 48, 64, 96, 128, 160, 200, 256, 320, 400, 480, 560, 640, 768, 896, 1024):
        if L < args.k:
            continue
        r = w["index"].search(w["queries"], k=args.k, l_value=L, with_stats=False)
        rec = recall_at(r.ids, w["gt"], args.k)
        sweep[L] = rec
        log(f"  L={L} recall@{args.k}={rec:.4f}")
        if rec >= args.target_recall:
            chosen = L
            break
    if chosen is None:
        chosen = max(sweep)
    else:
        # refine between the last L below the target and the first above it, in steps of 16
        below = max([l_ for l_ in sweep if l_ < chosen] or [chosen])
        for L in range(below + 16, chosen, 16):
            r = w["index"].search(w["queries"], k=args.k, l_value=L, with_stats=False)
            rec = recall_at(r.ids, w["gt"], args.k)
            sweep[L] = rec
            log(f"  L={L} recall@{args.k}={rec:.4f}")
            if rec >= args.target_recall:
                chosen = L
                break
    return chosen, sweep[chosen], sweep


def algorithmic_bytes(stats, D, M, rerank, k):
    """Bytes the search must read per query at their algorithmic size (device layout):
    per hop 4 + 4*deg adjacency; per gated neighbour D/8 MSB + 16 factor bytes; per scored
    survivor D/2 code + 16 header bytes; per reranked record 16 + D/2 + D/8 + D/2."""
    s = stats
    hops = s["hops"].astype(np.float64)
    gated = s["paper_msb_kernel_calls"].astype(np.float64)
    scored = s["paper_remaining_kernel_calls"].astype(np.float64)
    rer = float(max(rerank, k))
    per_q = hops * (4 + 4 * M) + gated * (D / 8 + 16) + scored * (D / 2 + 16) + rer * (16 + D / 2 + D / 8 + D / 2)
    return float(per_q.sum())


def oracle_index(w, n):
    """The index arrays on the host, in the layout the oracle's search reads."""
    def host(t):
        return t.cpu().numpy() if hasattr(t, "cpu") else np.asarray(t)

    return dict(compact=host(w["compact"]), residual=host(w["residual"]), msb=host(w["msb"]),
                factors=host(w["factors"]), degrees=host(w["deg"]).view(np.uint32),
                edges=host(w["edges"]).view(np.uint32), total_points=n, base_points=n)


def codec_ablation(torch, w, args, log):
    """The reference's ablation query codecs (rabitq_set_query_coarse_codec: Int4, B1, B1Main,
    Full) and the Int8 search with the opt-in fused rerank (RABITQ_ENABLE_FUSED_INT_RERANK)
    through the same index and queries as the Int8 headline: for each, the smallest L
    reaching the recall target (the headline's sweep), its device-timed QPS, and parity with the
    oracle searching with that codec on a sample of the queries (ids, distance bits, counters)."""
    from quantization_graph_gb300.space import CODEC_B1, CODEC_B1MAIN, CODEC_FULL, CODEC_INT4, CODEC_INT8

    codes = {"int4": CODEC_INT4, "b1": CODEC_B1, "b1main": CODEC_B1MAIN, "full": CODEC_FULL,
             "int8_fused": CODEC_INT8}  # the Int8 search with the opt-in fused restore + residual rerank
    names = [c.strip() for c in args.codecs.split(",") if c.strip()]
    if not names:
        return {}
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build()
    space, index, q = w["space"], w["index"], w["queries"]
    nq = q.shape[0]
    sweep_args = argparse.Namespace(**{**vars(args), "L": 0})
    ids = torch.empty((nq, args.k), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, args.k), dtype=torch.float32, device="cuda")
    stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
    center = space.center.cpu().numpy() if hasattr(space.center, "cpu") else space.center
    oindex = oracle_index(w, args.n)
    out = {}
    try:
        for name in names:
            space.set_query_coarse_codec(codes[name])
            fused = name.endswith("_fused")
            log(f"codec {name}:")
            L, rec, _ = pick_l(torch, w, sweep_args, log)
            index.search_into(q, ids, dists, k=args.k, l_value=L, stats_out=stats, fused_int_rerank=fused)
            torch.cuda.synchronize()
            if fused:
                rec = recall_at(ids.to(torch.int64), w["gt"], args.k)
            for _ in range(args.warmup):
                index.search_into(q, ids, dists, k=args.k, l_value=L, fused_int_rerank=fused)
            ms = device_ms(torch, lambda: index.search_into(q, ids, dists, k=args.k, l_value=L,
                                                            fused_int_rerank=fused), args.steps)
            index.search_into(q, ids, dists, k=args.k, l_value=L, stats_out=stats, fused_int_rerank=fused)
            torch.cuda.synchronize()
            count = min(nq, args.codec_parity_queries)
            sample = np.linspace(0, nq - 1, count).astype(np.int64)
            o = oracle_py.Oracle(args.dim, center, codec=codes[name])
            oi, od, ost = o.search(q.cpu().numpy()[sample], oindex, k=args.k, L=L, threads=os.cpu_count() or 1,
                                   fused=fused)
            gi = ids.cpu().numpy().view(np.uint32)[sample]
            gd = dists.cpu().numpy()[sample]
            gs = stats_struct(stats, nq)[sample]
            c_bad = np.zeros(count, bool)
            for f in gs.dtype.names:
                c_bad |= gs[f] != ost[f]
            out[name] = {"L": int(L), "recall@10": round(float(rec), 4), "qps": round(nq / ms * 1000.0, 1),
                         "ms_per_batch": round(ms, 3),
                         "parity": {"queries": int(count), "id_mismatch": int((~(gi == oi).all(1)).sum()),
                                    "dist_bit_mismatch": int((~(gd.view(np.uint32) == od.view(np.uint32)).all(1)).sum()),
                                    "counter_mismatch": int(c_bad.sum())}}
            log(f"  codec {name}: L={L} recall {rec:.4f}, {out[name]['qps']:.0f} QPS, parity {out[name]['parity']}")
    finally:
        space.set_query_coarse_codec(CODEC_INT8)
    return out


def cpu_parity(w, args, L, gpu_ids, gpu_dists, gpu_stats, log):
    """The reference search restated on the CPU (oracle/), all host threads, over a sample of the
    same queries at the same L: ids, distance bits and the 9 OursPaperSearchStats counters must
    equal the GPU's (the check of verify_search_parity, ours_diskann.rs:1988-2066). Its wall time
    is the CPU baseline. Returns (parity, cpu_baseline)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build()
    nq = gpu_ids.shape[0]
    count = min(nq, args.parity_queries)
    sample = np.linspace(0, nq - 1, count).astype(np.int64) if count < nq else np.arange(nq)
    o = oracle_py.Oracle(args.dim, w["space"].center.cpu().numpy() if hasattr(w["space"].center, "cpu")
                         else w["space"].center)
    index = oracle_index(w, args.n)
    q = w["queries"].cpu().numpy()[sample]
    threads = os.cpu_count() or 1
    t = time.time()
    oi, od, ost = o.search(q, index, k=args.k, L=L, threads=threads)
    el = time.time() - t
    gi = gpu_ids[sample].astype(np.uint32)
    gd = gpu_dists[sample].astype(np.float32)
    gs = gpu_stats[sample]
    id_bad = ~(gi == oi).all(1)
    d_bad = ~(gd.view(np.uint32) == od.view(np.uint32)).all(1)
    fields = gs.dtype.names
    c_bad = np.zeros(count, bool)
    for f in fields:
        c_bad |= gs[f] != ost[f]
    parity = {"queries": int(count), "L": int(L), "k": args.k, "id_mismatch": int(id_bad.sum()),
              "dist_bit_mismatch": int(d_bad.sum()), "counter_mismatch": int(c_bad.sum()),
              "counters": list(fields),
              "against": "the reference search restated on the CPU (oracle/qg_oracle.cpp), pinned to the "
                         "reference's own bridge; queries evenly spaced over the batch"}
    log(f"parity at L={L}: {count} queries, id {parity['id_mismatch']}, distance bits {parity['dist_bit_mismatch']}, "
        f"counters {parity['counter_mismatch']} mismatching; CPU {count / el:.1f} queries/s on {threads} threads")
    cpu = {"value": count / el, "unit": "queries/s", "cores": threads, "kind": "port",
           "sample": f"{count} of {nq} queries (evenly spaced) at L={L}, k={args.k}, one query per thread; "
                     "the same queries the parity check compares"}
    return parity, cpu


def encode_parity(w, args, log):
    """A seeded sample of base rows re-encoded by the oracle encoder (pinned to the reference's
    encodeVectorFullWithCentroid) and compared with the GPU's records."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build()
    n = w["compact"].shape[0]
    rows = np.sort(np.random.default_rng(11).choice(n, size=min(n, args.encode_parity_rows), replace=False))
    o = oracle_py.Oracle(args.dim, w["space"].center.cpu().numpy() if hasattr(w["space"].center, "cpu")
                         else w["space"].center)
    import torch

    ridx = torch.from_numpy(rows).cuda()
    X = w["base"][ridx].cpu().numpy()
    t = time.time()
    oc, orr = o.encode(X, threads=os.cpu_count() or 1)
    el = time.time() - t
    gc = w["compact"][ridx].cpu().numpy()
    gr = w["residual"][ridx].cpu().numpy()
    D = o.D
    codes_o = oc[:, 16:16 + D // 2]
    codes_g = gc[:, 16:16 + D // 2]
    nib_bad = int(((codes_o & 15) != (codes_g & 15)).sum() + ((codes_o >> 4) != (codes_g >> 4)).sum())
    fo = oc[:, :16].copy().view(np.float32).astype(np.float64)
    fg = gc[:, :16].copy().view(np.float32).astype(np.float64)
    rel = np.abs(fo - fg) / np.maximum(np.abs(fo), 1e-30)
    out = {"rows": int(len(rows)), "compact_records_equal": int((oc == gc).all(1).sum()),
           "residual_records_equal": int((orr == gr).all(1).sum()),
           "code_mismatch_rate": nib_bad / (len(rows) * D), "max_factor_rel_err": float(rel.max()),
           "against": "the oracle encoder (restated encodeVectorFullWithCentroid, pinned to the reference)",
           "oracle_seconds": round(el, 2)}
    log(f"encode parity: {out['compact_records_equal']}/{len(rows)} compact and {out['residual_records_equal']}"
        f"/{len(rows)} residual records byte-equal, code mismatch rate {out['code_mismatch_rate']:.2e}")
    return out


def device_ms(torch, fn, steps):
    """Mean device time of `fn` over `steps` calls (CUDA events on the current stream)."""
    stream = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(stream)
    for _ in range(steps):
        fn()
    end.record(stream)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / steps


def pipelined_ms(torch, fns, streams, steps):
    """Mean device time per step, step s issued by fns[s % n] on streams[s % n]: CUDA events on the
    current stream, which every stream waits on before the first step and which waits on every
    stream after the last, so the region covers all steps of all streams."""
    cur = torch.cuda.current_stream()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    start.record(cur)
    for st in streams:
        st.wait_event(start)
    for i in range(steps):
        j = i % len(fns)
        with torch.cuda.stream(streams[j]):
            fns[j]()
    for st in streams:
        cur.wait_stream(st)
    end.record(cur)
    torch.cuda.synchronize()
    return start.elapsed_time(end) / steps


def stats_struct(stats, nq):
    names = ("visited_nodes", "distance_computations", "hops", "paper_checked", "paper_would_prune",
             "paper_not_pruned", "paper_full_saved", "paper_msb_kernel_calls", "paper_remaining_kernel_calls")
    return stats.cpu().numpy().view(np.dtype([(f, "<u8") for f in names])).reshape(nq)


def learned_stop_select(torch, w, args, L_fixed, rec_fixed, log):
    """Train the stop networks on held-out queries (a stop classifier and a hop budget, from the
    same traces of the plain search) and pick the (model, L, knob) with the highest QPS whose
    recall is >= the target and within 0.002 of the plain fixed-L operating point."""
    import dataclasses

    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic

    index, q, gt = w["index"], w["queries"], w["gt"]
    cands = sorted({min(1024, max(args.k, int(round(L_fixed * f / 8.0)) * 8)) for f in (1.0, 1.25, 1.5, 2.0)})
    L_train = max(cands)
    t0 = time.time()
    # held-out queries from the base distribution of the workload
    if args.workload == "gist960":
        tq = synthetic.anisotropic_torch(args.train_queries, args.dim, 1.2, seed=3, absolute=True)
    else:
        tq = synthetic.anisotropic_torch(args.train_queries, args.dim, 0.8, seed=3, normalize=True)
    truth = index.search(tq, k=args.k, l_value=L_train, with_stats=False).ids.to(torch.int32)
    tr = ls.collect_traces(index, tq, truth, k=args.k, l_value=L_train, every=args.stop_every)
    h_star = tr.hops_needed().double()
    oracle_frac = float(h_star.sum() / tr.final_hops.double().sum())
    log(f"learned stop: {tr.features.shape[0]} trace rows from {args.train_queries} held-out queries at "
        f"L={L_train}; an oracle stop (each query at the first hop whose rerank window holds its final result) "
        f"needs {oracle_frac:.3f} of the hops")
    min_hops = 2 * args.stop_every
    models = {}
    if args.stop_kind in ("classifier", "both"):
        models["classifier"] = ls.train(tr.features, tr.classifier_labels(), epochs=args.stop_epochs,
                                        every=args.stop_every, min_hops=min_hops, log=log)
    if args.stop_kind in ("budget", "both"):
        keep = tr.hop >= min_hops  # the kernel predicts from min_hops on
        budget = ls.train(tr.features[keep], tr.budget_targets()[keep], epochs=args.stop_epochs,
                          every=args.stop_every, min_hops=min_hops, log=log, kind=ls.KIND_BUDGET)
        models["budget"] = budget
        models["budget-once"] = dataclasses.replace(budget, predict_once=True)
        # how much of log(h*) the network explains: over all rows, and at the first prediction
        y = tr.budget_targets()[keep]
        z = ls.forward(budget.weights, budget.norm, tr.features[keep])
        r2_rows = float(1.0 - ((z - y) ** 2).mean() / y.var())
        first = keep & (tr.hop == min_hops)
        y1 = tr.budget_targets()[first]
        z1 = ls.forward(budget.weights, budget.norm, tr.features[first])
        r2_first = float(1.0 - ((z1 - y1) ** 2).mean() / y1.var())
        log(f"  hop budget: R^2 of log(h*) {r2_rows:.3f} over the checkpoints, {r2_first:.3f} at hop {min_hops}")
    t_train = time.time() - t0
    del tq, tr, truth
    knobs = {"classifier": (0.5, 0.7, 0.8, 0.9, 0.95, 0.98, 0.99),
             "budget": (0.5, 0.7, 0.85, 1.0, 1.2, 1.5, 2.0), "budget-once": (0.7, 1.0, 1.5, 2.0, 3.0)}
    ids = torch.empty((q.shape[0], args.k), dtype=torch.int32, device="cuda")
    dists = torch.empty((q.shape[0], args.k), dtype=torch.float32, device="cuda")
    table = []
    best = None
    for L in cands:
        r = index.search(q, k=args.k, l_value=L, with_stats=False)
        rec_l = recall_at(r.ids, gt, args.k)
        fms = device_ms(torch, lambda: index.search_into(q, ids, dists, k=args.k, l_value=L), 2)
        for name, model in models.items():
            for knob in knobs[name]:
                ls.search(index, q, model, knob, k=args.k, l_value=L, ids_out=ids, dists_out=dists)
                rec = recall_at(ids.to(torch.int64), gt, args.k)
                ms = device_ms(torch, lambda: ls.search(index, q, model, knob, k=args.k, l_value=L, ids_out=ids,
                                                       dists_out=dists), 2)
                row = {"model": name, "L": L, "knob": knob, "recall": round(rec, 4),
                       "fixed_recall_same_L": round(rec_l, 4), "qps": round(q.shape[0] / ms * 1000.0, 1),
                       "fixed_qps_same_L": round(q.shape[0] / fms * 1000.0, 1)}
                table.append(row)
                ok = rec >= args.target_recall and rec >= rec_fixed - 0.002
                if ok and (best is None or ms < best["ms"]):
                    best = {"model": name, "L": L, "knob": knob, "ms": ms, "recall": rec,
                            "fixed_recall_same_L": rec_l}
            log(f"  L={L} {name}: fixed recall {rec_l:.4f}; " + ", ".join(
                f"{r_['knob']}: {r_['recall']:.4f}/{r_['qps']:.0f}" for r_ in table
                if r_["L"] == L and r_["model"] == name))

    def run(qq, ids_out, dists_out, stats_out=None, idx=index):
        ls.search(idx, qq, models[best["model"]], best["knob"], k=args.k, l_value=best["L"], ids_out=ids_out,
                  dists_out=dists_out, stats_out=stats_out)

    info = {"oracle_stop_hop_fraction": round(oracle_frac, 4), "train_L": L_train}
    if "budget" in models:
        info.update(budget_r2_checkpoints=round(r2_rows, 4), budget_r2_first_prediction=round(r2_first, 4))
    return best, table, t_train, run, info


def shard_range(nq: int, world: int, rank: int) -> tuple[int, int]:
    """Query ids [lo, hi) searched by `rank`: contiguous id ranges of (nearly) equal size."""
    return nq * rank // world, nq * (rank + 1) // world


def replica_aggregate(step_ms: float, e2e_ms: float, total_units: int, world: int, device="cuda"):
    """Query-sharded replicas: every rank times the search of its own query range; the job's step
    time is the slowest rank's (all_reduce MAX over the process group) and the job's throughput
    counts every query once. Returns (step_ms, e2e_ms, value, e2e_value)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([step_ms, e2e_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    step_ms, e2e_ms = float(t[0]), float(t[1])
    return step_ms, e2e_ms, total_units / (step_ms / 1000.0), total_units / (e2e_ms / 1000.0)


def gather_shards(local, nq: int, world: int):
    """All ranks' rows of a [rows of my shard, ...] tensor, in query-id order (every rank gets the
    whole [nq, ...] result). Shards are padded to the largest for the all_gather."""
    import torch
    import torch.distributed as dist

    if world == 1:
        return local
    width = (nq + world - 1) // world
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[:local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    return torch.cat([parts[r][:shard_range(nq, world, r)[1] - shard_range(nq, world, r)[0]] for r in range(world)])


def setup_cache(args, log):
    """The reference arm's set-up process: builds the workload's index on the GPU with this
    library, picks the operating L, and writes everything the timed CPU search reads."""
    import torch

    from quantization_graph_gb300 import build as qbuild

    qbuild.build()
    torch.cuda.set_device(0)
    w = build_workload(torch, args, log)
    L, rec, sweep = pick_l(torch, w, args, log)
    d = args.setup_cache
    host = oracle_index(w, args.n)
    for name in ("compact", "residual", "msb", "factors", "degrees", "edges"):
        np.save(os.path.join(d, f"{name}.npy"), host[name])
    np.save(os.path.join(d, "queries.npy"), w["queries"].cpu().numpy())
    np.save(os.path.join(d, "gt.npy"), w["gt"].cpu().numpy())
    center = w["space"].center
    np.save(os.path.join(d, "center.npy"), center.cpu().numpy() if hasattr(center, "cpu") else np.asarray(center))
    json.dump({"L": L, "recall_gpu": rec, "ground_truth": w["gt_info"]}, open(os.path.join(d, "meta.json"), "w"))


def reference_arm(args, log):
    """--impl reference: the reference search restated on the host cores (oracle/, all threads) at
    the same L over the same index and queries. Set-up runs in a child process (GPU index build,
    written to a temporary cache); this process loads only the oracle. Each step searches one
    slice of queries (one query per thread at a time) sized to --ref-step-seconds; value = the
    queries of the timed steps / their wall time (diskann_runner.rs:369-439: wall time of the
    search loop only)."""
    metric, config = workload_config(args)
    cache = tempfile.mkdtemp(prefix="qg_ref_index_")
    try:
        cmd = [sys.executable, os.path.abspath(__file__), "--setup-cache", cache, "--workload", args.workload,
               "--n", str(args.n), "--dim", str(args.dim), "--nq", str(args.nq), "--M", str(args.M),
               "--k", str(args.k), "--target-recall", str(args.target_recall), "--L", str(args.L),
               "--graph", args.graph, "--l-build", str(args.l_build), "--refine", str(args.refine),
               "--knn", str(args.knn), "--refine-l", str(args.refine_l)]
        env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK=os.environ.get("LOCAL_RANK", "0"))
        t0 = time.time()
        subprocess.run(cmd, check=True, env=env)
        t_setup = time.time() - t0
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py

        oracle_py.build()
        load = {name: np.load(os.path.join(cache, f"{name}.npy")) for name in
                ("compact", "residual", "msb", "factors", "degrees", "edges", "queries", "gt", "center")}
        meta = json.load(open(os.path.join(cache, "meta.json")))
    finally:
        shutil.rmtree(cache, ignore_errors=True)
    L = int(meta["L"])
    index = {k_: load[k_] for k_ in ("compact", "residual", "msb", "factors", "degrees", "edges")}
    index.update(total_points=args.n, base_points=args.n)
    q, gt = load["queries"], load["gt"]
    o = oracle_py.Oracle(args.dim, load["center"])
    threads = os.cpu_count() or 1
    t = time.perf_counter()
    o.search(q[:threads], index, k=args.k, L=L, threads=threads)
    per_round = time.perf_counter() - t  # one query per thread
    per_step = threads * max(1, int(round(args.ref_step_seconds / max(per_round, 1e-6))))
    per_step = min(per_step, q.shape[0])
    pos = threads
    ids_all, seen = [], []

    def step():
        nonlocal pos
        idx = (np.arange(pos, pos + per_step) % q.shape[0])
        pos += per_step
        r = o.search(q[idx], index, k=args.k, L=L, threads=threads)
        return idx, r[0]

    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        idx, ids = step()
        times.append(time.perf_counter() - t)
        ids_all.append(ids)
        seen.append(idx)
    total = sum(times)
    value = args.steps * per_step / total
    rec = recall_np(np.concatenate(ids_all), gt[np.concatenate(seen)], args.k)
    log(f"reference arm: {args.steps} steps of {per_step} queries at L={L} in {total:.2f}s on {threads} threads, "
        f"recall {rec:.4f}")
    cpu = {"value": value, "unit": "queries/s", "cores": threads, "kind": "port",
           "sample": f"{args.steps} steps of {per_step} queries (a slice of the {q.shape[0]} queries, one query per "
                     f"thread) at L={L}, k={args.k}"}
    line = {"impl": "reference", "metric": metric, "value": value, "unit": "queries/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int8/f32",
            "data": "synthetic", "config": config,
            "search": {"mode": "fixed-L (the reference has no learned stop)", "L": L, "recall@10": round(rec, 4),
                       "queries_per_step": per_step,
                       "implementation": "the reference's search loop and kernels restated in C++ (oracle/"
                                         "qg_oracle.cpp, pinned bit for bit to the reference's own bridge); the "
                                         "reference's own build is x86 AVX-512 C++ plus Rust and does not run on "
                                         "this host"},
            "setup": {"seconds": round(t_setup, 1), "process": "separate child process: index encoded and "
                      "graph built on the GPU by this library, cached to files; the timed process loads only "
                      "the oracle"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    def log(msg):
        if rank == 0:
            print(msg, file=sys.stderr, flush=True)

    if args.setup_cache:
        setup_cache(args, log)
        return
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args, log)
        return
    import torch
    import torch.distributed as dist

    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from quantization_graph_gb300 import build as qbuild

    qbuild.build()
    metric, config = workload_config(args)
    w = build_workload(torch, args, log)
    L, rec, sweep = pick_l(torch, w, args, log)
    log(f"fixed-L: L={L} recall={rec:.4f}")
    D = w["space"].code_dim
    index = w["index"]
    q = w["queries"]
    nq = q.shape[0]
    lo, hi = shard_range(nq, world, rank)
    ql = q[lo:hi].contiguous()
    nl = ql.shape[0]
    ids = torch.empty((nq, args.k), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, args.k), dtype=torch.float32, device="cuda")
    stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")

    # fixed-L over the whole batch: the fallback, the judge, and the results the parity leg checks
    index.search_into(q, ids, dists, k=args.k, l_value=L, stats_out=stats)
    torch.cuda.synchronize()
    fixed_ids = ids.cpu().numpy().view(np.uint32).copy()
    fixed_d = dists.cpu().numpy().copy()
    fixed_stats = stats_struct(stats, nq).copy()
    for _ in range(args.warmup):
        index.search_into(q, ids, dists, k=args.k, l_value=L)
    fixed_ms = device_ms(torch, lambda: index.search_into(q, ids, dists, k=args.k, l_value=L), args.steps)
    fixed = {"L": L, "recall@10": round(rec, 4), "qps": round(nq / fixed_ms * 1000.0, 1)}

    # learned stop
    search_info = {"fixed_l": fixed, "mode": "fixed-L", "L": L, "tile": args.tile, "launch": args.launch or "auto"}
    run_learned = None
    if not args.no_learned:
        best, table, t_train, run_learned, linfo = learned_stop_select(torch, w, args, L, rec, log)
        search_info["learned_stop_sweep"] = table
        search_info["learned_stop_train"] = dict(linfo, seconds=round(t_train, 1), queries=args.train_queries,
                                                 checkpoint_every_hops=args.stop_every)
        if best is not None:
            search_info["learned_stop"] = {"model": best["model"], "L": best["L"], "knob": best["knob"],
                                           "recall@10": round(best["recall"], 4),
                                           "fixed_recall_same_L": round(best["fixed_recall_same_L"], 4),
                                           "qps": round(nq / best["ms"] * 1000.0, 1),
                                           "vs_fixed_l": round(fixed_ms / best["ms"], 3),
                                           "criterion": "recall >= target and >= fixed-L operating point - 0.002"}
            if best["ms"] < fixed_ms:  # the headline takes whichever mode is faster at the target recall
                search_info.update(mode="learned-stop", L=best["L"], model=best["model"], knob=best["knob"])
        if search_info["mode"] != "learned-stop":
            run_learned = None

    def step(qq, ids_out, dists_out, stats_out=None, idx=index):
        if run_learned is not None:
            run_learned(qq, ids_out, dists_out, stats_out, idx=idx)
        else:
            idx.search_into(qq, ids_out, dists_out, k=args.k, l_value=L, stats_out=stats_out)

    # counters of the chosen mode over the whole batch, for the algorithmic bytes and the recall
    step(q, ids, dists, stats)
    torch.cuda.synchronize()
    final_recall = recall_at(ids.to(torch.int64), w["gt"], args.k)
    alg_bytes = algorithmic_bytes(stats_struct(stats, nq), D, args.M, 100, args.k)

    # the timed region: this rank's query range, `inflight` batches in flight (a handle on the
    # same resident index, outputs and a stream per slot)
    nf = max(1, args.inflight)
    handles = [index] + [index.share() for _ in range(nf - 1)]
    streams = [torch.cuda.Stream() for _ in range(nf)]
    ids_l = [torch.empty((nl, args.k), dtype=torch.int32, device="cuda") for _ in range(nf)]
    d_l = [torch.empty((nl, args.k), dtype=torch.float32, device="cuda") for _ in range(nf)]
    hq = ql.cpu().pin_memory()
    hid = [torch.empty((nl, args.k), dtype=torch.int32).pin_memory() for _ in range(nf)]
    hd = [torch.empty((nl, args.k), dtype=torch.float32).pin_memory() for _ in range(nf)]
    dq = [torch.empty_like(ql) for _ in range(nf)]

    def device_step(j):
        return lambda: step(ql, ids_l[j], d_l[j], idx=handles[j])

    def e2e_step(j):
        def fn():
            dq[j].copy_(hq, non_blocking=True)
            step(dq[j], ids_l[j], d_l[j], idx=handles[j])
            hid[j].copy_(ids_l[j], non_blocking=True)
            hd[j].copy_(d_l[j], non_blocking=True)
        return fn

    dev_fns = [device_step(j) for j in range(nf)]
    e2e_fns = [e2e_step(j) for j in range(nf)]
    for fns in (dev_fns, e2e_fns):  # every handle's scratch settled before the timed region
        pipelined_ms(torch, fns, streams, max(args.warmup, nf))
    for _ in range(args.warmup):
        step(ql, ids_l[0], d_l[0])
    prep_ms = device_ms(torch, lambda: w["space"].prepare(ql), args.steps)

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        # one launch at a time: the search kernel's own duration, for the roofline
        seq_ms = device_ms(torch, dev_fns[0], args.steps)
        step_ms = pipelined_ms(torch, dev_fns, streams, args.steps)
        e2e_ms = pipelined_ms(torch, e2e_fns, streams, args.steps)
    if world > 1:
        dist.barrier()
    seq_ms = replica_aggregate(seq_ms, seq_ms, nq, world)[0]
    step_ms, e2e_ms, value, e2e_value = replica_aggregate(step_ms, e2e_ms, nq, world)
    ok = all(bool((hid[j].to(torch.int64).cuda() == ids_l[j].to(torch.int64)).all()) and
             bool((ids_l[j] == ids_l[0]).all()) for j in range(min(nf, args.steps)))
    ids_l = ids_l[0]
    gathered = gather_shards(ids_l, nq, world)
    sharded_recall = recall_at(gathered.to(torch.int64), w["gt"], args.k)
    search_ms = max(seq_ms - prep_ms, 1e-6)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    alg_local = alg_bytes * nl / nq
    achieved = alg_local / (search_ms / 1000.0) / 1e9
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "search_kernel_traffic.json")))
        ratio = prof.get("dram_over_algorithmic")
        if ratio is not None:
            traffic = ratio * alg_local
    except (OSError, ValueError):
        pass
    parity, cpu, enc = None, None, None
    if rank == 0 and not args.skip_cpu:
        parity, cpu = cpu_parity(w, args, L, fixed_ids, fixed_d, fixed_stats, log)
        enc = encode_parity(w, args, log)
        if world == 1 and args.codecs:
            search_info["codecs"] = codec_ablation(torch, w, args, log)
    search_info.update({"recall@10": round(final_recall, 4), "recall@10_gathered_shards": round(sharded_recall, 4),
                        "queries_per_rank": nl, "l_sweep": {str(k_): round(v, 4) for k_, v in sweep.items()},
                        "inflight": nf,
                        "one_at_a_time": {"ms_per_step": round(seq_ms, 3), "qps": round(nq / seq_ms * 1000.0, 1)},
                        "timing": (f"value and e2e: {args.steps} steps of {nl} queries, {nf} in flight (a handle on "
                                   "the same resident index and a stream each, step s on slot s mod "
                                   f"{nf}); the roofline's kernel time: the same steps one at a time")})
    line = {"metric": metric, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8/f32", "data": "synthetic", "config": config,
            "search": search_info,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(nl * args.dim * 4),
                    "d2h_bytes_per_step": int(nl * args.k * 8), "results_match_device": ok},
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "search_kernel", "kernel_ms": search_ms, "prep_ms": prep_ms,
                         "algorithmic_bytes_per_query": alg_bytes / nq,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "clocks": clocks.summary(), "cpu_baseline": cpu, "parity": parity, "encode_parity": enc,
            "ground_truth": w["gt_info"],
            "setup": {"encode_s": round(w["t_encode"], 3), "graph_s": round(w["t_graph"], 2), "graph": args.graph,
                      "reachable_from_0": round(w["reach"], 5)}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    bad = parity is not None and (parity["id_mismatch"] or parity["dist_bit_mismatch"] or parity["counter_mismatch"])
    for c in search_info.get("codecs", {}).values():
        p_ = c["parity"]
        bad = bad or bool(p_["id_mismatch"] or p_["dist_bit_mismatch"] or p_["counter_mismatch"])
    if world > 1:
        dist.destroy_process_group()
    if bad:
        print("parity check failed: the GPU search differs from the reference restatement", file=sys.stderr)
        sys.exit(3)


def run_encode(args, log):
    """GPU encode of the 1M x 1536 unit-norm base two ways: the reference's rotation (random
    signs + fast Hadamard transform, bit-exact to the reference encoder) and the rotation as a
    BF16x3 GEMM on the tcgen05 tensor cores (qg_encode_batch_gemm). Reports the GEMM's time and
    throughput (useful FLOPs 2 N dim D, the three BF16 passes counted as overhead), the
    code-mismatch rate and factor error of the GEMM path against the reference encoder over all
    rows, and both rotations' error against an FP64 rotation on a row sample."""
    import torch

    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.space import RabitqSpace, train_global_center

    base = synthetic.anisotropic_torch(args.n, args.dim, 0.8, seed=1, normalize=True)
    space = RabitqSpace(args.dim, train_global_center(base))
    D = space.code_dim
    torch.cuda.synchronize()
    t = time.time()
    c_ref, r_ref = space.encode(base)
    torch.cuda.synchronize()
    t_fht = time.time() - t
    t = time.time()
    c_gem, r_gem = space.encode_gemm(base)
    torch.cuda.synchronize()
    t_gem = time.time() - t
    # the rotation alone, device-timed over chunks of 131072 rows (the GEMM entry point's chunk)
    chunk = min(args.n, 131072)
    rows = base[:chunk]
    for _ in range(max(1, args.warmup)):
        space.rotate_gemm(rows)
    ms = device_ms(torch, lambda: space.rotate_gemm(rows), max(1, args.steps))
    kp = (args.dim + 63) // 64 * 64
    useful = 2.0 * chunk * args.dim * D
    issued = 2.0 * chunk * 3 * kp * D
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("bf16_tflops", 1900.0))
    codes_r = c_ref[:, 16:16 + D // 2]
    codes_g = c_gem[:, 16:16 + D // 2]
    nib_bad = int(((codes_r & 15) != (codes_g & 15)).sum() + ((codes_r >> 4) != (codes_g >> 4)).sum())
    fr = c_ref[:, :16].contiguous().view(torch.float32).double()
    fg = c_gem[:, :16].contiguous().view(torch.float32).double()
    rel = (fr - fg).abs() / fr.abs().clamp_min(1e-30)
    res_bad = int((r_ref != r_gem).any(1).sum())
    # both rotations against FP64 on a sample of rows: exact u = r / |r|, exact +-1/sqrt(D) signs
    sample = torch.arange(0, args.n, max(1, args.n // 256), device="cuda")[:256]
    rot_g, norms = space.rotate_gemm(base[sample])
    sgn = torch.from_numpy(space.signs()).cuda()
    r32 = base[sample] - torch.from_numpy(space.center).cuda()[None, :]
    u32 = r32 * (1.0 / norms)[:, None]  # the encoder's fl(r * fl(1 / |r|))
    fht = torch.nn.functional.pad(u32 * sgn[None, :args.dim], (0, D - args.dim))
    step = 1
    while step < D:  # the reference's butterflies in FP32 (space_rabitq.h:944-988)
        v = fht.view(-1, D // (2 * step), 2, step)
        fht = torch.stack((v[:, :, 0] + v[:, :, 1], v[:, :, 0] - v[:, :, 1]), 2).reshape(-1, D)
        step *= 2
    j_ = torch.arange(D, device="cuda")
    x = j_[:, None] & j_[None, :]
    for sh in (16, 8, 4, 2, 1):
        x = x ^ (x >> sh)
    H = 1.0 - 2.0 * (x & 1).double()
    r64 = r32.double() / r32.double().norm(dim=1, keepdim=True)
    s64 = torch.where(sgn > 0, 1.0, -1.0).double() / float(np.sqrt(D))
    exact = torch.nn.functional.pad(r64 * s64[None, :args.dim], (0, D - args.dim)) @ H.T
    scale = exact.abs().max()
    line = {"metric": "encode: rotation as a BF16x3 tcgen05 GEMM, 1M×1536 unit-norm (ExRaBitQ4 block16)",
            "value": useful / (ms / 1000.0) / 1e12, "unit": "TFLOP/s (useful, 2*N*dim*D)", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3/f32", "data": "synthetic",
            "config": {"workload": f"{args.n} x {args.dim} unit-norm anisotropic (lambda_i ~ i^-0.8), D={D}",
                       "gemm_rows_per_step": chunk, "k": 3 * kp},
            "roofline": {"bound": "tensor", "achieved": issued / (ms / 1000.0) / 1e12, "peak": peak,
                         "unit": "TFLOP/s", "frac": issued / (ms / 1000.0) / 1e12 / peak, "traffic": None,
                         "kernel": "rotate_gemm_kernel (+ rotate_split_kernel in the timed call)",
                         "note": "achieved counts the three BF16 passes (issued FLOPs); value counts useful FLOPs",
                         "peak_source": "MEASURED_PEAKS.json bf16_tflops (of measured)" if peaks else "fallback"},
            "encode": {"rows": args.n, "fht_encode_s": round(t_fht, 3), "gemm_encode_s": round(t_gem, 3),
                       "code_mismatch_rate": nib_bad / (args.n * D),
                       "compact_records_equal": int((c_ref == c_gem).all(1).sum()),
                       "residual_records_differing": res_bad,
                       "factor_rel_err": {"median": float(rel[:, 1:].median()), "max": float(rel[:, 1:].max()),
                                          "norm_sqr_max": float(rel[:, 0].max())},
                       "against": "the reference encoder (the FHT path, bit-exact to the reference)"},
            "rotation_error_vs_fp64": {"rows": int(sample.numel()), "max_abs_value": float(scale),
                                       "gemm_max_abs": float((rot_g.double() - exact).abs().max()),
                                       "fht_max_abs": float((fht.double() - exact).abs().max()),
                                       "gemm_vs_fht_max_abs": float((rot_g - fht).abs().max())}}
    log(f"encode: FHT {t_fht:.2f}s, GEMM path {t_gem:.2f}s; rotation GEMM {ms:.2f} ms per {chunk} rows "
        f"({line['value']:.0f} useful TFLOP/s); code mismatch {line['encode']['code_mismatch_rate']:.2e}")
    print(json.dumps(line), flush=True)


def run_stream(args, log):
    """Uneven batched stream: 200k queries over a 120k x 1024 clustered unit-norm index (16
    clusters, lambda_i ~ i^-1.0 within each), batch sizes log-uniform in [1, 4096], per-query
    k in {1, 10, 100} and L uniform in [20, 400]; every batch is one replay of the captured
    CUDA graph (GraphSearcher, several in flight through SearchPool) with the autotuned launch
    shape. Reports QPS over the whole
    stream and p50/p99 batch latency, measured end to end from pinned host buffers (queries,
    k and L copied in, ids copied out, per batch)."""
    import torch

    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.graph_build import build_graph, build_vamana, reachable_fraction
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace, train_global_center
    from quantization_graph_gb300.stream import SearchPool, autotune

    dim, n, nq_total = 1024, args.stream_n, args.stream_queries
    t0 = time.time()
    base = synthetic.clustered_torch(n, dim, 16, 1.0, seed=1)
    queries = synthetic.clustered_torch(nq_total, dim, 16, 1.0, seed=2)
    space = RabitqSpace(dim, train_global_center(base))
    compact, residual = space.encode(base)
    msb, factors = space.export_paper_sidecar(compact)
    if args.graph == "reference":
        deg, edges, _ = build_vamana(space, compact, r=args.M, l_build=args.l_build, alpha=1.2, beam=1, batch=4096,
                                     refine=args.refine, cap=256, stop_hops=2)
    else:
        deg, edges = build_graph(space, base, compact, r=args.M, knn=2 * args.M, alpha=1.2, reverse=args.M,
                                 refine_rounds=args.refine, refine_l=128, residual=residual, msb=msb, factors=factors)
    index = OursIndex(space, compact, residual, msb, factors, deg, edges)
    gt, gt_info = ground_truth(torch, base, queries, 10)
    torch.cuda.synchronize()
    t_setup = time.time() - t0
    log(f"stream setup {t_setup:.1f}s, reachable {reachable_fraction(edges):.4f}")

    rng = np.random.default_rng(5)
    sizes = []
    left = nq_total
    while left > 0:
        b = int(np.exp(rng.uniform(0.0, np.log(4097.0))))
        b = max(1, min(b, 4096, left))
        sizes.append(b)
        left -= b
    kq = rng.choice(np.array([1, 10, 100], np.int32), size=nq_total)
    lq = rng.integers(20, 401, size=nq_total).astype(np.int32)

    chk = index.search(queries[:4096], k=10, l_value=200, with_stats=False)
    log(f"plain search, 4096 queries, L=200: recall@10 {recall_at(chk.ids, gt[:4096], 10):.4f}")
    best, tune = autotune(index, queries[:4096], k=10, l_value=200, log=log)
    thresholds = [float(x) for x in args.stream_thresholds.split(",") if x.strip()]
    model = None
    if thresholds:
        # traces of the plain search over the stream's own mix of k and L (held-out queries)
        tq = synthetic.clustered_torch(24000, dim, 16, 1.0, seed=3)
        feats, labels, j = [], [], 0
        for kk in (1, 10, 100):
            for ll in (50, 100, 200, 400):
                sub = tq[j:j + 2000]
                j += 2000
                lv = max(ll, kk)
                truth = index.search(sub, k=kk, l_value=lv, with_stats=False).ids.to(torch.int32)
                tr = ls.collect_traces(index, sub, truth, k=kk, l_value=lv, every=args.stop_every)
                feats.append(tr.features)
                labels.append(tr.classifier_labels())
        model = ls.train(torch.cat(feats), torch.cat(labels), epochs=args.stop_epochs, every=args.stop_every,
                         min_hops=2 * args.stop_every, log=log)
        del tq, feats, labels
    hq = queries.cpu().pin_memory()
    hk = torch.from_numpy(kq).pin_memory()
    hl = torch.from_numpy(lq).pin_memory()
    out = torch.empty((nq_total, 100), dtype=torch.int32).pin_memory()
    k10 = torch.from_numpy(kq >= 10)
    k1 = torch.from_numpy(kq == 1)
    gtc = gt.cpu()

    bounds = np.concatenate([[0], np.cumsum(sizes)])
    batches = [(hq[a:b], hk[a:b], hl[a:b]) for a, b in zip(bounds[:-1], bounds[1:])]

    def measure(thr):
        pool = SearchPool(index, dim, max_batch=4096, max_k=100, max_l=400, inflight=args.stream_inflight,
                          model=model if thr else None, threshold=thr)
        pool.run(batches, out)  # warm-up pass over the whole stream
        with ClockSampler(0) as clocks:
            lat, elapsed = pool.run(batches, out)
        ids_all = out.to(torch.int64)
        hit = (ids_all[k10][:, :10, None] == gtc[k10][:, None, :10]).any(-1).sum().item()
        rec10 = hit / (int(k10.sum()) * 10)
        rec1 = (ids_all[k1][:, 0] == gtc[k1][:, 0]).float().mean().item()
        lat_a = np.array(lat)
        r = {"threshold": thr, "qps": nq_total / elapsed, "recall@10 (k>=10 queries)": round(rec10, 4),
             "recall@1 (k=1 queries)": round(rec1, 4),
             "batch_latency_ms": {"p50": float(np.percentile(lat_a, 50)), "p99": float(np.percentile(lat_a, 99)),
                                  "max": float(lat_a.max())}, "ms_per_batch": float(lat_a.mean()),
             "clocks": clocks.summary()}
        log(f"  stream {'fixed L' if not thr else f'learned stop t={thr}'}: {r['qps']:.0f} qps, "
            f"recall@10 {rec10:.4f}, recall@1 {rec1:.4f}, p50 {r['batch_latency_ms']['p50']:.2f} ms, "
            f"p99 {r['batch_latency_ms']['p99']:.2f} ms")
        del pool
        return r

    fixed = measure(None)
    modes = [fixed] + [measure(t) for t in thresholds]
    # the headline: the fastest mode whose recall@10 is >= 0.95 and within 0.002 of fixed L
    ok = [m for m in modes if m["recall@10 (k>=10 queries)"] >= 0.95 and
          m["recall@10 (k>=10 queries)"] >= fixed["recall@10 (k>=10 queries)"] - 0.002]
    best_mode = max(ok or [fixed], key=lambda m: m["qps"])
    line = {"metric": "QPS, uneven batched stream, 120k\u00d71024 clustered 4-bit, 1 GB300",
            "value": best_mode["qps"], "unit": "queries/s", "n_gpus": 1, "steps": len(sizes), "warmup": len(sizes),
            "ms_per_step": best_mode["ms_per_batch"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8/f32", "data": "synthetic",
            "config": {"workload": (f"{n} x {dim} unit-norm 16-cluster mixture (lambda_i ~ i^-1.0, centre spread = "
                                    f"within-cluster spread), M={args.M}, {nq_total} queries in {len(sizes)} batches "
                                    "(log-uniform 1..4096), k in {1,10,100}, L ~ U[20,400]"),
                       "launch": {"warps_per_block": best[0], "blocks_per_sm": best[1] or "max", "tile": best[2],
                                  "tuned": [[list(s_), round(ms, 3)] for s_, ms in tune]},
                       "mode": "fixed per-query L" if not best_mode["threshold"] else
                               f"learned stop, threshold {best_mode['threshold']}",
                       "recall@10 (k>=10 queries)": best_mode["recall@10 (k>=10 queries)"],
                       "recall@1 (k=1 queries)": best_mode["recall@1 (k=1 queries)"],
                       "batch_latency_ms": best_mode["batch_latency_ms"],
                       "modes": [{k_: v for k_, v in m.items() if k_ != "clocks"} for m in modes],
                       "inflight": args.stream_inflight,
                       "timing": (f"up to {args.stream_inflight} batches in flight (SearchPool: a handle and a stream "
                                  "each); QPS = queries / wall time of the whole stream; batch latency = device "
                                  "time on the batch's stream from its pinned H2D of queries/k/L through the graph "
                                  "replay to the D2H of its ids")},
            "e2e": {"value": best_mode["qps"], "unit": "queries/s",
                    "h2d_bytes_per_step": int(nq_total * (dim * 4 + 8) / len(sizes)),
                    "d2h_bytes_per_step": int(nq_total * 400 / len(sizes))},
            "gpu_launches": 2 * len(sizes), "clocks": best_mode["clocks"],
            "setup": {"seconds": round(t_setup, 1)}, "ground_truth": gt_info}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    _args = parse()
    if _args.workload in ("stream", "encode"):
        from quantization_graph_gb300 import build as _qb

        _qb.build()
        (run_stream if _args.workload == "stream" else run_encode)(_args, lambda m: print(m, file=sys.stderr,
                                                                                           flush=True))
    else:
        main()
