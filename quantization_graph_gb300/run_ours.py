"""Run the Ours-DiskANN method for one dataset on the GPU: the host driver that
Ours/experiments/run_ours.py (:142-224) and the runner it spawns (run_diskann_fair,
experiments/02_diskann_fair/src/diskann_runner.rs:155-551, run_ours_exrabitq4) make together.

    python -m quantization_graph_gb300.run_ours --dataset dbpedia --M 32,64

Per degree: the 03 shared query split (first --val-queries queries validation, the rest test;
run_ours.py:36-101), base vectors from <data-root>/<dataset>/<dataset>_base.fvecs, the global
centre (diskann_runner.rs:1677-1701), GPU ExRaBitQ4 encode, the graph -- loaded from
<out-root>/02_diskann_fair/<dataset>/indexes/Ours/<dataset>_Ours_R<M>_Lbuild400.graph.bin when it
exists (run_ours.py:209-222: the frozen formal graph), otherwise built by the reference's Vamana
algorithm on the GPU (build beam 400, alpha 1.2, --refine-passes, prune cap 256, early stop 2)
and saved there -- the paper-prune sidecar, then a sweep of search list sizes with the
reference's timing protocol (diskann_runner.rs:369-439: wall time of the searches only, `repeats`
passes over the test queries, recall@10 against the ground truth, the offline FP32 accuracy
audit outside the timed region), appending one diskann_fair_raw.csv row per L in the reference's
schema and keeping only the latest formal INT8 row per L (keep_only_formal_int8_rows,
run_ours.py:104-139).

The GPU searches a batch of queries per launch: qps = queries / wall time of the launches;
latency_mean_us / latency_p95_us are the mean and 95th percentile over the repeats of one batch's
wall time (the latency a query sees when it is submitted with its batch).
"""
from __future__ import annotations

import argparse
import csv
import os
import time
from pathlib import Path

import numpy as np

from . import graph_io, runio

CODECS = {"full": 0, "b1": 1, "int4": 2, "int8": 3, "b1main": 4, "full-staged": 5, "full-rerank-scalar": 6}
DEFAULT_L = [10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28, 29, 30, 40, 50, 60, 70, 80,
             90, 100, 140, 180, 220, 260, 300, 340, 380, 420, 460]  # args.rs:52-55


def keep_only_formal_int8_rows(csv_path, degree: int) -> None:
    """Keeps every row but this degree's Ours rows, and of those only the latest INT8 row per
    search list size (run_ours.py:104-139)."""
    csv_path = Path(csv_path)
    if not csv_path.exists():
        return
    with csv_path.open(newline="") as handle:
        lines = [ln for ln in handle if not ln.startswith("#")]
    reader = csv.DictReader(lines)
    fieldnames = list(reader.fieldnames or [])
    rows = list(reader)
    if not rows:
        return
    preserved, latest = [], {}
    for row in rows:
        if not (row.get("method") == "Ours" and int(row.get("max_degree", 0) or 0) == degree):
            preserved.append(row)
            continue
        if row.get("query_coarse_codec", "").strip('"').lower() == "int8":
            latest[int(row.get("search_param_value", 0) or 0)] = row
    if not latest:
        raise RuntimeError(f"formal INT8 run produced no Ours rows with max_degree={degree}: {csv_path}")
    tmp = csv_path.with_suffix(csv_path.suffix + ".tmp")
    with tmp.open("w", newline="") as handle:
        writer = csv.DictWriter(handle, fieldnames=fieldnames, lineterminator="\n")
        writer.writeheader()
        writer.writerows(preserved)
        writer.writerows(row for _, row in sorted(latest.items()))
    tmp.replace(csv_path)


def graph_path(out_root, dataset: str, degree: int) -> Path:
    return Path(out_root) / "02_diskann_fair" / dataset / "indexes" / "Ours" / f"{dataset}_Ours_R{degree}_Lbuild400.graph.bin"


def run_degree(args, degree: int, test_q: np.ndarray, test_gt: np.ndarray, base: np.ndarray, log=print) -> list:
    import torch

    from .graph_build import build_vamana
    from .index import OursIndex
    from .space import RabitqSpace, train_global_center

    t_all = time.time()
    dev = torch.from_numpy(base).cuda()
    t0 = time.time()
    center = train_global_center(dev, sample_count=args.centroid_train_samples)
    space = RabitqSpace(base.shape[1], center, codec=CODECS[args.query_coarse_codec])
    torch.cuda.synchronize()
    train_ms = (time.time() - t0) * 1e3
    t0 = time.time()
    compact, residual = space.encode(dev)
    torch.cuda.synchronize()
    encode_ms = (time.time() - t0) * 1e3
    gfile = Path(args.graph_file) if args.graph_file else graph_path(args.out_root, args.dataset, degree)
    t0 = time.time()
    if gfile.exists():
        deg, edges, _, _, _ = graph_io.load_graph(str(gfile))
        mode = f"loaded {gfile.name}"
        evals = None
    else:
        d, e, evals = build_vamana(space, compact, r=degree, l_build=args.build_beam, alpha=args.alpha, beam=1,
                                   batch=args.build_batch_size, refine=args.refine_passes, cap=256, stop_hops=2)
        deg = d.cpu().numpy().view(np.uint32)
        edges = e.cpu().numpy().view(np.uint32)
        gfile.parent.mkdir(parents=True, exist_ok=True)
        graph_io.save_graph(str(gfile), deg, edges)
        # the runner's frozen start point, as the file holds it: adjacency [0] (ours_diskann.rs:2144-2146)
        deg = np.concatenate([deg, np.array([1], np.uint32)])
        edges = np.concatenate([edges, np.zeros((1, edges.shape[1]), np.uint32)])
        mode = "built on the GPU (the reference's Vamana algorithm)"
    total = len(deg)
    torch.cuda.synchronize()
    graph_ms = (time.time() - t0) * 1e3
    msb, factors = space.export_paper_sidecar(compact)
    index = OursIndex(space, compact, residual, msb, factors, deg, edges, base_points=base.shape[0],
                      total_points=total)
    build_ms = (time.time() - t_all) * 1e3
    log(f"R={degree}: encode {encode_ms:.0f} ms, graph {graph_ms:.0f} ms ({mode}), index "
        f"{index.device_bytes() / 1e6:.1f} MB on the device")

    q = torch.from_numpy(np.ascontiguousarray(test_q)).cuda()
    nq = q.shape[0]
    k = 10
    ids = torch.empty((nq, k), dtype=torch.int32, device="cuda")
    dists = torch.empty((nq, k), dtype=torch.float32, device="cuda")
    stats = torch.empty((nq, 9), dtype=torch.int64, device="cuda")
    results = []
    for L in args.search_list_sizes:
        index.search_into(q, ids, dists, k=k, l_value=L, stats_out=stats)  # warm-up
        torch.cuda.synchronize()
        lat = []
        t_search = time.perf_counter()
        for _ in range(args.repeats):
            t1 = time.perf_counter()
            index.search_into(q, ids, dists, k=k, l_value=L, stats_out=stats)
            torch.cuda.synchronize()
            lat.append((time.perf_counter() - t1) * 1e6)
        elapsed = time.perf_counter() - t_search
        got = ids.cpu().numpy().view(np.uint32).astype(np.int64)
        got_d = dists.cpu().numpy()
        hits = sum(runio.recall_hits(got[i], test_gt[i][:k]) for i in range(nq))
        audit = runio.AccuracyAudit()
        for i in range(nq):  # offline, outside the timed region
            audit.add(got[i], got_d[i], test_q[i], base, test_gt[i][:k])
        res = dict(search_list_size=L, query_coarse_codec=args.query_coarse_codec, recall=hits / (nq * k),
                   qps=nq * args.repeats / max(elapsed, 1e-12), latency_mean_us=float(np.mean(lat)),
                   latency_p95_us=runio.percentile(lat, 0.95), ffi_calls_per_query=1.0 / nq)
        res.update(runio.stats_per_query(stats.cpu().numpy()))
        res.update(audit.summary())
        results.append(res)
        log(f"  L={L}: recall@10 {res['recall']:.4f}, {res['qps']:.0f} queries/s")
    run = dict(dataset=args.dataset, method="Ours", status="done", graph_build_distance="ExRaBitQ4 symmetric",
               graph_build_mode=mode, graph_build_distance_evaluations=evals, max_degree=degree,
               build_beam=args.build_beam, alpha=args.alpha, search_beam_width=1, threads=1, seed=20260813,
               encode_time_ms=encode_ms, train_time_ms=train_ms, graph_build_time_ms=graph_ms,
               build_time_ms=build_ms, index_bytes=index.device_bytes(),
               index_size_mb=index.device_bytes() / (1024.0 * 1024.0), fp32_base_bytes=0,
               actual_bytes_per_vector=(space.compact_record_bytes() + space.residual_record_bytes()),
               log_path=str(log_path(args.out_root, args.dataset, degree)),
               note=("Ours ExRaBitQ4 block16 on one GB300: GPU encode, the reference's Vamana graph, batched "
                     "paper-prune INT8 search and residual4 rerank in one kernel launch per batch; latency is the "
                     "batch wall time"))
    return run, results


def log_path(out_root, dataset: str, degree: int) -> Path:
    return Path(out_root) / "02_diskann_fair" / dataset / "logs" / "Ours" / f"{dataset}_Ours_R{degree}_Lbuild400.log"


def write_log(path: Path, run: dict, results: list) -> None:
    path.parent.mkdir(parents=True, exist_ok=True)
    with path.open("w") as f:
        f.write("suite=02_diskann_fair\n")
        for key in sorted(run):
            f.write(f"{key}={run[key]}\n")
        for res in results:
            f.write("result " + " ".join(f"{k}={v}" for k, v in res.items()) + "\n")


def parse(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--dataset", required=True)
    ap.add_argument("--M", default="32,64", help="comma-separated max-degree values (32 and/or 64)")
    ap.add_argument("--data-root", default="data")
    ap.add_argument("--out-root", default=os.path.join("results", "memory_environment"))
    ap.add_argument("--val-queries", type=int, default=1000)
    ap.add_argument("--repeats", type=int, default=1)
    ap.add_argument("--graph-file", default="", help="use this graph instead of the per-degree formal graph")
    ap.add_argument("--query-coarse-codec", default="int8", choices=list(CODECS))
    ap.add_argument("--search-list-sizes", default=",".join(str(x) for x in DEFAULT_L))
    ap.add_argument("--refine-passes", type=int, default=2, help="03 end-to-end keeps refine 2 (run_ours.py:198-200)")
    ap.add_argument("--build-beam", type=int, default=400)
    ap.add_argument("--alpha", type=float, default=1.2)
    ap.add_argument("--build-batch-size", type=int, default=32768,
                    help="nodes inserted per bulk batch (the runner's default, args.rs:63); a batch's searches see "
                         "the graph as it was at the batch start, so a batch near n gives a poor graph on small data")
    ap.add_argument("--centroid-train-samples", type=int, default=100_000)
    args = ap.parse_args(argv)
    args.degrees = [int(v) for v in args.M.split(",") if v.strip()]
    if not args.degrees or any(d not in (32, 64) for d in args.degrees):
        ap.error("--M values must be 32 or 64")
    args.search_list_sizes = [int(v) for v in args.search_list_sizes.split(",") if v.strip()]
    return args


def main(argv=None) -> int:
    args = parse(argv)
    _, _, test_q_path, test_gt_path = runio.prepare_query_splits(args.dataset, args.data_root, args.out_root,
                                                                 args.val_queries)
    test_q = runio.read_fvecs(test_q_path)
    test_gt = runio.read_ivecs(test_gt_path)
    base = runio.read_fvecs(Path(args.data_root) / args.dataset / f"{args.dataset}_base.fvecs")
    csv_path = Path(args.out_root) / "02_diskann_fair" / args.dataset / "csv" / "diskann_fair_raw.csv"
    for degree in args.degrees:
        run, results = run_degree(args, degree, test_q, test_gt, base)
        runio.append_raw_csv(csv_path, run, results)
        write_log(log_path(args.out_root, args.dataset, degree), run, results)
        if args.query_coarse_codec == "int8":
            keep_only_formal_int8_rows(csv_path, degree)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
