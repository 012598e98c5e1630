#!/usr/bin/env python
"""Benchmark: QPS at recall@10 >= 0.95 of the Ours-DiskANN query path on one GB300.

Workload (default): 1,000,000 base vectors x 1536-d, unit-norm anisotropic Gaussian
(lambda_i ~ i^-0.8, seeded rotation), 10,000 queries drawn the same way, ExRaBitQ4 block16
encoding on the GPU, degree-64 graph built by the reference's Vamana algorithm on the GPU
(rabitq_build_vamana_graph with the formal arguments: L_build 400, alpha 1.2, batch 4096, refine
1, prune cap 256, early stop 2; the same graph the reference builds; --graph own selects this
library's faster kNN + prune builder), k = 10, INT8 query codec with the 1-bit paper-prune gate,
residual4 top-100 rerank, fixed-L beam search with the smallest L from a sweep that reaches
recall@10 >= 0.95 against an exact FP64 ground truth.

One step = one batched search of all queries (one qg_search_batch: query preparation +
persistent search kernel). `value` is device-timed with inputs resident in HBM; `e2e` adds the
pinned host->device copy of the queries and the device->host copy of ids and distances.
The index (~2.6 GB) exceeds the 129 MB L2, so no flush is needed between steps.

--impl reference times the reference's search on the host cores instead (the CPU restatement
of the reference, oracle/, all threads), on the same index and queries.
Multi-GPU (torchrun): replicas only -- each rank searches its own copy; value sums ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


def parse():
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
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--graph", default="reference", choices=["reference", "own"],
                    help="reference: the reference's Vamana build (rabitq_build_vamana_graph) on the GPU with the "
                         "formal arguments; own: this library's kNN + prune builder")
    ap.add_argument("--l-build", type=int, default=400, help="build search list size (--graph reference)")
    ap.add_argument("--refine", type=int, default=1, help="graph refinement rounds")
    ap.add_argument("--knn", type=int, default=240, help="kNN candidates per node for the graph")
    ap.add_argument("--refine-l", type=int, default=256, help="search list size of the refinement rounds")
    ap.add_argument("--no-learned", action="store_true", help="fixed-L only")
    ap.add_argument("--train-queries", type=int, default=20_000)
    ap.add_argument("--stop-every", type=int, default=8)
    ap.add_argument("--stop-epochs", type=int, default=4)
    ap.add_argument("--workload", default="dbpedia1536", choices=["dbpedia1536", "gist960", "stream"],
                    help="gist960: 1M x 960 |x| with lambda_i ~ i^-1.2; stream: uneven batched stream over "
                         "a 120k x 1024 clustered index")
    ap.add_argument("--stream-n", type=int, default=120_000)
    ap.add_argument("--stream-queries", type=int, default=200_000)
    ap.add_argument("--stream-thresholds", default="0.9,0.95,0.98",
                    help="learned-stop thresholds tried on the stream ('' = fixed per-query L only)")
    return ap.parse_args()


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


def ground_truth(torch, base, queries, k):
    """Exact top-k: FP32 GEMM shortlist of 64 per query, re-scored in FP64."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        bn = (base * base).sum(1)
        short = []
        for s in range(0, queries.shape[0], 1024):
            q = queries[s:s + 1024]
            d = torch.addmm(bn[None, :], q, base.T, beta=1.0, alpha=-2.0)
            short.append(torch.topk(d, 64, dim=1, largest=False).indices)
        short = torch.cat(short)
        out = torch.empty((queries.shape[0], k), dtype=torch.int64, device=base.device)
        for s in range(0, queries.shape[0], 1024):
            cand = short[s:s + 1024]
            diff = base[cand].double() - queries[s:s + 1024, None, :].double()
            dd = (diff * diff).sum(-1)
            order = torch.argsort(dd, dim=1, stable=True)[:, :k]
            out[s:s + 1024] = torch.gather(cand, 1, order)
        return out
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def recall_at(ids, gt, k):
    hit = (ids[:, :k, None] == gt[:, None, :k]).any(-1).sum().item()
    return hit / (ids.shape[0] * k)


def graph_desc(args) -> str:
    if args.graph == "reference":
        return (f"the reference's Vamana build (rabitq_build_vamana_graph) on the GPU, identical graph: R={args.M}, "
                f"L_build={args.l_build}, alpha 1.2, beam 1, batch 4096, refine {args.refine}, prune cap 256, "
                f"early stop 2")
    return (f"GPU kNN-{args.knn or 2 * args.M} + 16 random + alpha-1.2 prune + reverse edges + "
            f"{args.refine} search-based refinement round(s) at L={args.refine_l}")


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
    gt = ground_truth(torch, base, queries, args.k)
    index = OursIndex(space, compact, residual, msb, factors, deg, edges)
    torch.cuda.empty_cache()
    log(f"setup: data {t1 - t0:.1f}s encode {t_encode:.2f}s graph {t_graph:.1f}s reachable {reach:.4f} "
        f"index {index.device_bytes() / 1e9:.2f} GB")
    return dict(base=base, queries=queries, space=space, index=index, gt=gt, compact=compact,
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


def cpu_baseline(w, args, L, log, steps=1, warmup=0):
    """Reference search restated on the CPU (oracle/), all host threads, bounded sample: `warmup`
    untimed rounds of one query per thread, then `steps` timed slices of a sample of about
    --cpu-seconds of work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py

    oracle_py.build()
    o = oracle_py.Oracle(args.dim, w["space"].center)
    index = dict(compact=w["compact"].cpu().numpy(), residual=w["residual"].cpu().numpy(),
                 msb=w["msb"].cpu().numpy(), factors=w["factors"].cpu().numpy(),
                 degrees=w["deg"].cpu().numpy().view(np.uint32), edges=w["edges"].cpu().numpy().view(np.uint32),
                 total_points=args.n, base_points=args.n)
    q = w["queries"].cpu().numpy()
    threads = os.cpu_count() or 1
    t = time.time()
    o.search(q[:threads * 4], index, k=args.k, L=L, threads=threads)
    per = (time.time() - t) / (threads * 4)
    for i in range(warmup):
        o.search(q[i * threads:(i + 1) * threads], index, k=args.k, L=L, threads=threads)
    count = int(min(len(q), max(threads * 8, args.cpu_seconds / max(per, 1e-6))))
    steps = max(1, min(steps, count // threads))
    bounds = np.linspace(0, count, steps + 1).astype(int)
    el = 0.0
    parts = []
    for a_, b_ in zip(bounds[:-1], bounds[1:]):
        t = time.time()
        part, _, _ = o.search(q[a_:b_], index, k=args.k, L=L, threads=threads)
        el += time.time() - t
        parts.append(part)
    ids = np.concatenate(parts)
    gt = w["gt"][:count].cpu().numpy()
    rec = float(np.mean([len(set(a) & set(b)) / args.k for a, b in zip(ids, gt)]))
    log(f"cpu oracle: {count} queries in {el:.2f}s on {threads} threads, recall {rec:.4f}")
    return {"value": count / el, "unit": "queries/s", "cores": threads, "kind": "port", "steps": steps,
            "sample": f"{count} of {len(q)} queries at L={L}, k={args.k}, one query per thread"}, rec


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


def stats_struct(stats, nq):
    names = ("visited_nodes", "distance_computations", "hops", "paper_checked", "paper_would_prune",
             "paper_not_pruned", "paper_full_saved", "paper_msb_kernel_calls", "paper_remaining_kernel_calls")
    return stats.cpu().numpy().view(np.dtype([(f, "<u8") for f in names])).reshape(nq)


def learned_stop_select(torch, w, args, L_fixed, rec_fixed, log):
    """Train the stop network on held-out queries and pick (L, threshold) with the highest QPS
    whose recall is >= the target and within 0.002 of fixed-L at the same L."""
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
    feats, labels = ls.collect_traces(index, tq, truth, k=args.k, l_value=L_train, every=args.stop_every)
    log(f"learned stop: {feats.shape[0]} trace rows from {args.train_queries} held-out queries at L={L_train}, "
        f"positive {float(labels.mean()):.3f}")
    model = ls.train(feats, labels, epochs=args.stop_epochs, every=args.stop_every, min_hops=2 * args.stop_every,
                     log=log)
    t_train = time.time() - t0
    del tq, feats, labels, truth
    ids = torch.empty((q.shape[0], args.k), dtype=torch.int32, device="cuda")
    dists = torch.empty((q.shape[0], args.k), dtype=torch.float32, device="cuda")
    table = []
    best = None
    for L in cands:
        r = index.search(q, k=args.k, l_value=L, with_stats=False)
        rec_l = recall_at(r.ids, gt, args.k)
        fixed_ms = device_ms(torch, lambda: index.search_into(q, ids, dists, k=args.k, l_value=L), 2)
        for thr in (0.5, 0.7, 0.8, 0.9, 0.95, 0.98, 0.99):
            ls.search(index, q, model, thr, k=args.k, l_value=L, ids_out=ids, dists_out=dists)
            rec = recall_at(ids.to(torch.int64), gt, args.k)
            ms = device_ms(torch, lambda: ls.search(index, q, model, thr, k=args.k, l_value=L, ids_out=ids,
                                                   dists_out=dists), 2)
            row = {"L": L, "threshold": thr, "recall": round(rec, 4), "fixed_recall": round(rec_l, 4),
                   "qps": round(q.shape[0] / ms * 1000.0, 1), "fixed_qps": round(q.shape[0] / fixed_ms * 1000.0, 1)}
            table.append(row)
            ok = rec >= args.target_recall and rec >= rec_l - 0.002
            if ok and (best is None or ms < best[2]):
                best = (L, thr, ms, rec, rec_l)
        log(f"  L={L}: fixed recall {rec_l:.4f}; " + ", ".join(
            f"t={r_['threshold']}: {r_['recall']:.4f}/{r_['qps']:.0f}" for r_ in table if r_["L"] == L))
    return model, best, table, t_train


def replica_aggregate(step_ms: float, e2e_ms: float, units_per_rank: int, world: int, device="cuda"):
    """Replicas only: every rank times its own copy of the workload; the job's step time is the
    slowest rank's (all_reduce MAX over the process group) and the job's throughput counts every
    rank's units. Returns (step_ms, e2e_ms, value, e2e_value)."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([step_ms, e2e_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    step_ms, e2e_ms = float(t[0]), float(t[1])
    return step_ms, e2e_ms, world * units_per_rank / (step_ms / 1000.0), world * units_per_rank / (e2e_ms / 1000.0)


def main():
    args = parse()
    if args.workload == "gist960" and args.dim == 1536:
        args.dim = 960
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference" and rank != 0:
        return
    if world > 1 and args.impl == "ours":
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    def log(msg):
        if rank == 0:
            print(msg, file=sys.stderr, flush=True)

    from quantization_graph_gb300 import build as qbuild
    from quantization_graph_gb300 import learned_stop as ls

    qbuild.build()
    w = build_workload(torch, args, log)
    L, rec, sweep = pick_l(torch, w, args, log)
    log(f"fixed-L: L={L} recall={rec:.4f}")
    metric = "QPS@recall10=0.95, 1M\u00d71536 4-bit, learned-stop vs fixed-L beam, 1 GB300"
    data_desc = f"{args.n} x {args.dim} unit-norm anisotropic (lambda_i ~ i^-0.8)"
    if args.workload == "gist960":
        metric = "QPS@recall10=0.95, 1M\u00d7960 4-bit, fixed-L beam, 1 GB300"
        data_desc = f"{args.n} x {args.dim} |x|, x ~ N(0, Q diag(i^-1.2) Q^T)"
    config = {"workload": (f"{data_desc}, M={args.M}, "
                           f"{args.nq} queries, k={args.k}, INT8 paper-prune gate, residual4 rerank 100"),
              "n": args.n, "dim": args.dim, "queries": args.nq, "M": args.M, "k": args.k,
              "graph": graph_desc(args),
              "l2": "index larger than L2 (no flush needed)",
              "fixed_l": {"L": L, "recall@10": round(rec, 4)}}
    D = w["space"].code_dim

    if args.impl == "reference":
        cpu, cpu_rec = cpu_baseline(w, args, L, log, steps=args.steps, warmup=args.warmup)
        config["fixed_l"]["recall_cpu"] = round(cpu_rec, 4)
        line = {"impl": "reference", "metric": metric, "value": cpu["value"], "unit": "queries/s", "n_gpus": 1,
                "steps": cpu["steps"], "warmup": args.warmup, "ms_per_step": 1000.0 * args.nq / cpu["value"],
                "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int8/f32", "data": "synthetic",
                "config": dict(config, mode="fixed-L on the host cores (the reference search has no learned stop)"),
                "cpu_baseline": cpu,
                "e2e": {"value": cpu["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    index = w["index"]
    q = w["queries"]
    nq = q.shape[0]
    ids = torch.empty((nq, args.k), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, args.k), dtype=torch.float32, device="cuda")
    stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")

    # fixed-L: the fallback and the judge
    for _ in range(args.warmup):
        index.search_into(q, ids, dists, k=args.k, l_value=L)
    fixed_ms = device_ms(torch, lambda: index.search_into(q, ids, dists, k=args.k, l_value=L), args.steps)
    config["fixed_l"]["qps"] = round(world * nq / fixed_ms * 1000.0, 1)

    # learned stop
    mode = {"kind": "fixed-L", "L": L, "threshold": None}
    table, t_train, model = [], 0.0, None
    if not args.no_learned:
        model, best, table, t_train = learned_stop_select(torch, w, args, L, rec, log)
        if best is not None:
            config["learned_stop"] = {"L": best[0], "threshold": best[1], "recall@10": round(best[3], 4),
                                      "fixed_recall_same_L": round(best[4], 4),
                                      "qps": round(world * nq / best[2] * 1000.0, 1), "train_s": round(t_train, 1),
                                      "train_queries": args.train_queries, "checkpoint_every_hops": args.stop_every}
            # the headline takes whichever mode is faster at the target recall
            if best[2] < fixed_ms:
                mode = {"kind": "learned-stop", "L": best[0], "threshold": best[1]}
        config["learned_stop_sweep"] = table

    def step(qq):
        if mode["kind"] == "learned-stop":
            ls.search(index, qq, model, mode["threshold"], k=args.k, l_value=mode["L"], ids_out=ids, dists_out=dists)
        else:
            index.search_into(qq, ids, dists, k=args.k, l_value=mode["L"])

    # counters of the chosen mode, for the algorithmic bytes
    if mode["kind"] == "learned-stop":
        ls.search(index, q, model, mode["threshold"], k=args.k, l_value=mode["L"], ids_out=ids, dists_out=dists,
                  stats_out=stats)
    else:
        index.search_into(q, ids, dists, k=args.k, l_value=L, stats_out=stats)
    torch.cuda.synchronize()
    final_recall = recall_at(ids.to(torch.int64), w["gt"], args.k)
    alg_bytes = algorithmic_bytes(stats_struct(stats, nq), D, args.M, 100, args.k)
    for _ in range(args.warmup):
        step(q)
    prep_ms = device_ms(torch, lambda: w["space"].prepare(q), args.steps)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        step_ms = device_ms(torch, lambda: step(q), args.steps)
        # end to end through the public API with host buffers
        hq = q.cpu().pin_memory()
        hid = torch.empty((nq, args.k), dtype=torch.int32).pin_memory()
        hd = torch.empty((nq, args.k), dtype=torch.float32).pin_memory()
        dq = torch.empty_like(q)

        def e2e_step():
            dq.copy_(hq, non_blocking=True)
            step(dq)
            hid.copy_(ids, non_blocking=True)
            hd.copy_(dists, non_blocking=True)

        e2e_ms = device_ms(torch, e2e_step, args.steps)
    step_ms, e2e_ms, value, e2e_value = replica_aggregate(step_ms, e2e_ms, nq, world)
    ok = bool((hid.to(torch.int64).cuda() == ids.to(torch.int64)).all())
    search_ms = max(step_ms - prep_ms, 1e-6)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = alg_bytes / (search_ms / 1000.0) / 1e9
    traffic = None
    try:
        prof = json.load(open(os.path.join(ROOT, "profiles", "search_kernel_traffic.json")))
        ratio = prof.get("dram_over_algorithmic")
        if ratio is not None:
            traffic = ratio * alg_bytes
    except (OSError, ValueError):
        pass
    cpu = None
    if rank == 0 and not args.skip_cpu:
        cpu, _ = cpu_baseline(w, args, L, log)
    config.update(mode=mode, **{"recall@10": round(final_recall, 4)})
    line = {"metric": metric, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "int8/f32", "data": "synthetic", "config": config,
            "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": int(nq * args.dim * 4),
                    "d2h_bytes_per_step": int(nq * args.k * 8), "results_match_device": ok},
            "gpu_launches": 2 * args.steps,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "search_kernel", "kernel_ms": search_ms, "prep_ms": prep_ms,
                         "algorithmic_bytes_per_query": alg_bytes / nq,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"},
            "clocks": clocks.summary(), "cpu_baseline": cpu,
            "setup": {"encode_s": round(w["t_encode"], 3), "graph_s": round(w["t_graph"], 2), "graph": args.graph,
                      "reachable_from_0": round(w["reach"], 5),
                      "l_sweep": {str(k): round(v, 4) for k, v in sweep.items()}}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_stream(args, log):
    """Uneven batched stream: 200k queries over a 120k x 1024 clustered unit-norm index (16
    clusters, lambda_i ~ i^-1.0 within each), batch sizes log-uniform in [1, 4096], per-query
    k in {1, 10, 100} and L uniform in [20, 400]; every batch is one replay of the captured
    CUDA graph (GraphSearcher) with the autotuned launch shape. Reports QPS over the whole
    stream and p50/p99 batch latency, measured end to end from pinned host buffers (queries,
    k and L copied in, ids copied out, per batch)."""
    import torch

    from quantization_graph_gb300 import learned_stop as ls
    from quantization_graph_gb300 import synthetic
    from quantization_graph_gb300.graph_build import build_graph, build_vamana, reachable_fraction
    from quantization_graph_gb300.index import OursIndex
    from quantization_graph_gb300.space import RabitqSpace, train_global_center
    from quantization_graph_gb300.stream import GraphSearcher, autotune

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
    gt = ground_truth(torch, base, queries, 10)
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
                f, lab = ls.collect_traces(index, sub, truth, k=kk, l_value=lv, every=args.stop_every)
                feats.append(f)
                labels.append(lab)
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

    def measure(thr):
        gs = GraphSearcher(index, dim, max_batch=4096, max_k=100, max_l=400, model=model if thr else None,
                           threshold=thr)

        def run():
            lat = []
            start = 0
            t_all = time.perf_counter()
            for b in sizes:
                tb = time.perf_counter()
                with torch.cuda.stream(gs.stream):
                    dq = hq[start:start + b].to("cuda", non_blocking=True)
                    dk = hk[start:start + b].to("cuda", non_blocking=True)
                    dl = hl[start:start + b].to("cuda", non_blocking=True)
                ids, _ = gs.search(dq, dk, dl)
                with torch.cuda.stream(gs.stream):
                    out[start:start + b].copy_(ids, non_blocking=True)
                gs.synchronize()
                lat.append((time.perf_counter() - tb) * 1000.0)
                start += b
            return lat, time.perf_counter() - t_all

        run()  # warm-up pass over the whole stream
        with ClockSampler(0) as clocks:
            lat, elapsed = run()
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
        del gs
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
                       "launch": {"warps_per_block": best[0], "blocks_per_sm": best[1] or "max",
                                  "tuned": [[list(s_), round(ms, 3)] for s_, ms in tune]},
                       "mode": "fixed per-query L" if not best_mode["threshold"] else
                               f"learned stop, threshold {best_mode['threshold']}",
                       "recall@10 (k>=10 queries)": best_mode["recall@10 (k>=10 queries)"],
                       "recall@1 (k=1 queries)": best_mode["recall@1 (k=1 queries)"],
                       "batch_latency_ms": best_mode["batch_latency_ms"],
                       "modes": [{k_: v for k_, v in m.items() if k_ != "clocks"} for m in modes],
                       "timing": "host wall clock per batch: pinned H2D of queries/k/L, graph replay, D2H of ids"},
            "e2e": {"value": best_mode["qps"], "unit": "queries/s",
                    "h2d_bytes_per_step": int(nq_total * (dim * 4 + 8) / len(sizes)),
                    "d2h_bytes_per_step": int(nq_total * 400 / len(sizes))},
            "gpu_launches": 2 * len(sizes), "clocks": best_mode["clocks"],
            "setup": {"seconds": round(t_setup, 1)}}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    _args = parse()
    if _args.workload == "stream":
        from quantization_graph_gb300 import build as _qb

        _qb.build()
        run_stream(_args, lambda m: print(m, file=sys.stderr, flush=True))
    else:
        main()
