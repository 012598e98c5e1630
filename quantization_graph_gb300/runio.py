"""Host IO and reporting of the reference's runs, so GPU results slot into its pipeline unchanged.

- fvecs / ivecs files: read_fvecs (read_fvecs_matrix, experiments/02_diskann_fair/src/
  diskann_runner.rs:1847-1889), read_ivecs_topk (:1891-1920), and the writers of
  Ours/experiments/run_ours.py:76-89.
- the shared query split of experiment 03 (first N queries validation, the rest test;
  run_ours.py:36-101): prepare_query_splits.
- recall and the offline FP32 accuracy audit (recall_hits, percentile, AccuracyAudit;
  diskann_runner.rs:1922-1930, 2002-2093).
- rows of diskann_fair_raw.csv in the reference's schema and number formatting
  (append_raw_csv, logging.rs:313-411), which the 03 adapter (experiments/03_system_fair/
  adapters/ours_adapter.py:26-79) reads unchanged.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np


# ------------------------------------------------------------------------------------------
# fvecs / ivecs
# ------------------------------------------------------------------------------------------
def read_fvecs(path) -> np.ndarray:
    """[n, dim] float32; every row's dimension must be positive and equal (the Rust reader's
    errors), a truncated last row is an error."""
    raw = np.fromfile(path, dtype="<u1")
    if raw.size == 0:
        return np.zeros((0, 0), np.float32)
    dim = int(raw[:4].view("<i4")[0])
    if dim <= 0:
        raise ValueError(f"{path} has invalid fvecs dim {dim}")
    row = 4 * (dim + 1)
    if raw.size % row:
        raise ValueError(f"{path} is truncated or its fvecs dimension changes")
    n = raw.size // row
    rec = raw.reshape(n, row)
    dims = rec[:, :4].copy().view("<i4")[:, 0]
    if np.any(dims != dim):
        bad = int(np.nonzero(dims != dim)[0][0])
        raise ValueError(f"{path} fvecs dimension changed from {dim} to {int(dims[bad])}")
    return rec[:, 4:].copy().view("<f4").reshape(n, dim).astype(np.float32)


def read_ivecs_topk(path, k: int) -> np.ndarray:
    """[n, k] uint32: the first k ids of every row; a row shorter than k is an error."""
    out = []
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if not head:
                break
            if len(head) < 4:
                raise ValueError(f"{path} is truncated")
            width = int(np.frombuffer(head, "<i4")[0])
            if width < k:
                raise ValueError(f"{path} groundtruth k={width} is smaller than requested recall@{k}")
            body = f.read(4 * width)
            if len(body) < 4 * width:
                raise ValueError(f"{path} is truncated")
            out.append(np.frombuffer(body, "<i4")[:k].astype(np.uint32))
    return np.vstack(out) if out else np.zeros((0, k), np.uint32)


def read_ivecs(path) -> np.ndarray:
    """All rows (equal widths), int64, as run_ours.py's reader returns them."""
    rows = []
    with open(path, "rb") as f:
        while True:
            head = f.read(4)
            if not head:
                break
            width = int(np.frombuffer(head, "<i4")[0])
            rows.append(np.frombuffer(f.read(width * 4), "<i4").astype(np.int64))
    return np.vstack(rows) if rows else np.zeros((0, 0), np.int64)


def write_fvecs(path, arr) -> None:
    arr = np.ascontiguousarray(arr, dtype="<f4")
    n, dim = arr.shape
    rec = np.empty((n, dim + 1), "<f4")
    rec[:, 0] = np.array([dim], "<i4").view("<f4")[0]
    rec[:, 1:] = arr
    rec.tofile(path)


def write_ivecs(path, arr) -> None:
    arr = np.ascontiguousarray(arr, dtype="<i4")
    n, width = arr.shape
    rec = np.empty((n, width + 1), "<i4")
    rec[:, 0] = width
    rec[:, 1:] = arr
    rec.tofile(path)


def prepare_query_splits(dataset: str, data_root, out_root, val_queries: int):
    """The 03 shared split: the first val_queries queries (and ground-truth rows) are the
    validation set, the rest the test set, written once under
    out_root/03_system_fair/<dataset>/csv/_query_splits/ and reused afterwards. Returns the
    paths (validation queries, validation gt, test queries, test gt)."""
    split = Path(out_root) / "03_system_fair" / dataset / "csv" / "_query_splits"
    split.mkdir(parents=True, exist_ok=True)
    paths = (split / "validation_query.fvecs", split / "validation_gt.ivecs", split / "test_query.fvecs",
             split / "test_gt.ivecs")
    if paths[3].exists():
        return paths
    queries = read_fvecs(Path(data_root) / dataset / f"{dataset}_query.fvecs")
    gt = read_ivecs(Path(data_root) / dataset / f"{dataset}_groundtruth.ivecs")
    n_val = min(val_queries, len(queries))
    write_fvecs(paths[0], queries[:n_val])
    write_ivecs(paths[1], gt[:n_val])
    write_fvecs(paths[2], queries[n_val:])
    write_ivecs(paths[3], gt[n_val:])
    return paths


# ------------------------------------------------------------------------------------------
# recall and the accuracy audit
# ------------------------------------------------------------------------------------------
def recall_hits(ids, gt) -> int:
    """Returned ids found in the query's ground-truth row."""
    g = set(int(x) for x in np.asarray(gt).ravel())
    return sum(1 for x in np.asarray(ids).ravel() if int(x) in g)


def percentile(values, p: float) -> float:
    """values sorted, then the entry at round((n - 1) p), half away from zero."""
    v = np.sort(np.asarray(values, np.float64))
    return float(v[int(math.floor((len(v) - 1) * p + 0.5))])


def exact_l2_sqr(query, vector) -> np.float32:
    """sum of (q_i - v_i)^2 in f32, accumulated in order (no FMA), as exact_l2_sqr."""
    d = np.asarray(query, np.float32) - np.asarray(vector, np.float32)
    return np.cumsum(d * d, dtype=np.float32)[-1] if d.size else np.float32(0.0)


@dataclass
class AccuracyAudit:
    """The offline FP32 audit of returned (id, distance) lists (AccuracyTotals)."""

    rel_errors: list = field(default_factory=list)
    abs_error_sum: float = 0.0
    overlap: int = 0
    evaluated: int = 0
    flipped_pairs: int = 0
    total_pairs: int = 0

    def add(self, ids, distances, query, base, gt) -> None:
        ids = np.asarray(ids)
        distances = np.asarray(distances, np.float32)
        n = min(len(ids), len(distances))
        if n == 0:
            return
        gset = set(int(x) for x in np.asarray(gt).ravel())
        exact = np.empty(n, np.float32)
        for i in range(n):
            e = exact_l2_sqr(query, base[int(ids[i])])
            exact[i] = e
            rep, ex = float(distances[i]), float(e)
            self.rel_errors.append(abs(rep - ex) / ex if ex > 1e-12 else 0.0)
            self.abs_error_sum += abs(rep - ex)
            self.evaluated += 1
            self.overlap += int(int(ids[i]) in gset)
        for i in range(n):
            for j in range(i + 1, n):
                self.total_pairs += 1
                self.flipped_pairs += int((distances[i] <= distances[j]) != (exact[i] <= exact[j]))

    def summary(self) -> dict:
        count = max(self.evaluated, 1)
        if self.rel_errors:
            mean_rel = sum(self.rel_errors) / len(self.rel_errors)
            srt = sorted(self.rel_errors)
            rank = int(math.ceil(len(srt) * 0.95))
            p95 = srt[min(max(rank, 1), len(srt)) - 1]
        else:
            mean_rel = p95 = float("nan")
        return dict(mean_relative_error=mean_rel, p95_relative_error=p95,
                    mean_absolute_error=self.abs_error_sum / count, top10_overlap=self.overlap / count,
                    pairwise_flip_rate_top10=(self.flipped_pairs / self.total_pairs if self.total_pairs
                                              else float("nan")))


# ------------------------------------------------------------------------------------------
# diskann_fair_raw.csv
# ------------------------------------------------------------------------------------------
RAW_CSV_HEADER = (
    "suite,dataset,method,status,graph_build_distance,graph_build_mode,graph_build_distance_evaluations,"
    "shared_graph_build_time_ms,metric,k,nominal_bpd,actual_bytes_per_vector,codebook_bytes,index_size_mb,"
    "index_bytes,auxiliary_bytes,residual_bytes,fp32_base_bytes,peak_rss_mb,build_time_ms,graph_build_time_ms,"
    "train_time_ms,encode_time_ms,max_degree,build_beam,alpha,search_param_name,search_param_value,"
    "search_beam_width,query_coarse_codec,recall,qps,latency_mean_us,latency_p95_us,prepare_us,traverse_us,"
    "rerank_us,neighbor_fetch_us,visited_mark_us,paper_batch_us,flush_us,visited_nodes,distance_calls,"
    "mean_relative_error,p95_relative_error,mean_absolute_error,top10_overlap,pairwise_flip_rate_top10,"
    "paper_checked,paper_would_prune,paper_msb_kernel_calls,paper_remaining_kernel_calls,ffi_calls_per_query,"
    "payload_bytes_read,avg_bits_read,refine_calls,threads,repeat_id,seed,log_path,note")


def peak_rss_mb() -> float | None:
    """VmHWM of this process in MB, as the reference's peak_rss_mb (diskann_runner.rs:2095-2105)."""
    try:
        with open("/proc/self/status") as f:
            for line in f:
                if line.startswith("VmHWM:"):
                    return float(line.split()[1]) / 1024.0
    except OSError:
        pass
    return None


def _f6(v) -> str:  # fmt_metric / format!("{:.6}")
    return "NaN" if v is None or (isinstance(v, float) and math.isnan(v)) else f"{float(v):.6f}"


def _opt_f(v) -> str:  # opt_f64
    return "" if v is None else f"{float(v):.6f}"


def _opt_u(v) -> str:  # opt_u64
    return "" if v is None else str(int(v))


def _quote(s: str) -> str:  # csv_quote
    return '"' + str(s).replace('"', '""') + '"'


def _f32_str(x: float) -> str:  # f32::to_string: the shortest decimal that reads back
    return str(np.float32(x))


def raw_csv_line(run: dict, res: dict) -> str:
    """One row: `run` holds the per-index fields (dataset, method, status, graph_*, sizes,
    times, max_degree, build_beam, alpha, search_beam_width, threads, seed, log_path, note),
    `res` one search point (search_list_size, query_coarse_codec, recall, qps, latencies,
    per-query stage times and counters, the accuracy summary). Absent optional fields print
    empty, absent metrics NaN, as the reference does."""
    g = run.get
    r = res.get
    cols = [
        "02_diskann_fair", g("dataset"), g("method", "Ours"), g("status", "done"),
        g("graph_build_distance", ""), g("graph_build_mode", ""), _opt_u(g("graph_build_distance_evaluations")),
        _opt_f(g("shared_graph_build_time_ms")), "L2", "10", "4", _opt_f(g("actual_bytes_per_vector")),
        _opt_u(g("codebook_bytes")), _opt_f(g("index_size_mb")), _opt_u(g("index_bytes")),
        _opt_u(g("auxiliary_bytes")), _opt_u(g("residual_bytes")), _opt_u(g("fp32_base_bytes")),
        _opt_f(g("peak_rss_mb", peak_rss_mb())), _opt_f(g("build_time_ms")), _opt_f(g("graph_build_time_ms")),
        _opt_f(g("train_time_ms")), _opt_f(g("encode_time_ms")), str(int(g("max_degree"))),
        str(int(g("build_beam"))), _f32_str(g("alpha", 1.2)), "efSearch", str(int(r("search_list_size"))),
        str(int(g("search_beam_width", 1))), _quote(r("query_coarse_codec", "int8")),
        f"{float(r('recall')):.6f}", f"{float(r('qps')):.6f}", f"{float(r('latency_mean_us')):.6f}",
        f"{float(r('latency_p95_us')):.6f}",
    ]
    for key in ("prepare_us", "traverse_us", "rerank_us", "neighbor_fetch_us", "visited_mark_us", "paper_batch_us",
                "flush_us", "visited_nodes", "distance_calls", "mean_relative_error", "p95_relative_error",
                "mean_absolute_error", "top10_overlap", "pairwise_flip_rate_top10", "paper_checked",
                "paper_would_prune", "paper_msb_kernel_calls", "paper_remaining_kernel_calls",
                "ffi_calls_per_query"):
        cols.append(_f6(r(key, float("nan"))))
    cols += ["NaN", "NaN", "0", str(int(g("threads", 1))), "aggregate", str(int(g("seed", 20260813))),
             str(g("log_path", "")), _quote(g("note", ""))]
    return ",".join(str(c) for c in cols)


def append_raw_csv(path, run: dict, results: list) -> None:
    """Appends rows; writes the header to a new file, and a schema reset line plus the header
    when an existing file starts with another header (logging.rs:319-345)."""
    path = Path(path)
    needs = not path.exists()
    matches = True
    if not needs:
        with open(path) as f:
            matches = f.readline().rstrip("\n") == RAW_CSV_HEADER
    os.makedirs(path.parent, exist_ok=True)
    with open(path, "a") as f:
        if needs or not matches:
            if not needs:
                f.write("# schema_reset=02_diskann_fair_real_metrics\n")
            f.write(RAW_CSV_HEADER + "\n")
        for res in results:
            f.write(raw_csv_line(run, res) + "\n")


def stats_per_query(stats) -> dict:
    """Per-query means of the nine search counters in the CSV's columns (stats: [nq, 9] in
    the OursPaperSearchStats order of qg_search_batch)."""
    s = np.asarray(stats, np.float64)
    m = s.mean(0) if len(s) else np.full(9, np.nan)
    return dict(visited_nodes=m[0], distance_calls=m[1], paper_checked=m[3], paper_would_prune=m[4],
                paper_msb_kernel_calls=m[7], paper_remaining_kernel_calls=m[8])
