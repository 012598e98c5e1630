"""Host IO and reporting (quantization_graph_gb300/runio.py) against the reference's own Python:
the 03 query split written by run_ours.py's prepare_query_splits, and the 03 adapter's reader of
diskann_fair_raw.csv rows (ours_adapter.py:26-79). Both are executed from the reference tree
when it is present (in this container); the rest checks the readers, the audit and the row
format on their own."""
import ast
import csv
import importlib.util
import math
import os
from pathlib import Path
from typing import Any

import numpy as np
import pytest

from quantization_graph_gb300 import runio

REF = os.environ.get("REF_ROOT", "/root/reference")


def _ref_function(path, name, extra=None):
    """One top-level function of a reference module, executed from its source (its module
    imports packages that are not in the tree)."""
    src = open(path).read()
    tree = ast.parse(src)
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == name)
    ns = {"csv": csv, "Path": Path, "Any": Any, "__builtins__": __builtins__}
    ns.update(extra or {})
    exec(compile(ast.Module(body=[fn], type_ignores=[]), path, "exec"), ns)
    return ns[name]


def test_fvecs_ivecs_round_trip_and_errors(tmp_path):
    rng = np.random.default_rng(0)
    x = rng.standard_normal((37, 19)).astype(np.float32)
    g = rng.integers(0, 1000, (37, 100)).astype(np.int32)
    runio.write_fvecs(tmp_path / "a.fvecs", x)
    runio.write_ivecs(tmp_path / "a.ivecs", g)
    np.testing.assert_array_equal(runio.read_fvecs(tmp_path / "a.fvecs"), x)
    np.testing.assert_array_equal(runio.read_ivecs(tmp_path / "a.ivecs"), g)
    np.testing.assert_array_equal(runio.read_ivecs_topk(tmp_path / "a.ivecs", 10), g[:, :10].astype(np.uint32))
    with pytest.raises(ValueError):
        runio.read_ivecs_topk(tmp_path / "a.ivecs", 101)  # rows shorter than k
    raw = (tmp_path / "a.fvecs").read_bytes()
    (tmp_path / "t.fvecs").write_bytes(raw[:-4])
    with pytest.raises(ValueError):
        runio.read_fvecs(tmp_path / "t.fvecs")
    bad = bytearray(raw)
    bad[4 * 20:4 * 21] = np.array([18], "<i4").tobytes()  # second row's dimension
    (tmp_path / "d.fvecs").write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        runio.read_fvecs(tmp_path / "d.fvecs")


@pytest.mark.skipif(not os.path.isdir(REF), reason="needs the reference tree")
def test_query_split_matches_reference(tmp_path):
    spec = importlib.util.spec_from_file_location("run_ours", f"{REF}/Ours/experiments/run_ours.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rng = np.random.default_rng(1)
    data = tmp_path / "data" / "toy"
    data.mkdir(parents=True)
    runio.write_fvecs(data / "toy_query.fvecs", rng.standard_normal((300, 24)).astype(np.float32))
    runio.write_ivecs(data / "toy_groundtruth.ivecs", rng.integers(0, 5000, (300, 100)).astype(np.int32))
    theirs = mod.prepare_query_splits("toy", tmp_path / "data", tmp_path / "ref", 100)
    ours = runio.prepare_query_splits("toy", tmp_path / "data", tmp_path / "ours", 100)
    for a, b in zip(theirs, ours):
        assert a.name == b.name and a.read_bytes() == b.read_bytes()


def test_accuracy_audit_restated():
    rng = np.random.default_rng(2)
    base = rng.standard_normal((50, 33)).astype(np.float32)
    q = rng.standard_normal(33).astype(np.float32)
    ids = rng.permutation(50)[:10]
    exact = np.array([runio.exact_l2_sqr(q, base[i]) for i in ids], np.float32)
    # sequential f32 accumulation, as exact_l2_sqr does
    for i, idx in enumerate(ids):
        s = np.float32(0)
        for a, b in zip(q, base[idx]):
            d = np.float32(a - b)
            s = np.float32(s + np.float32(d * d))
        assert s == exact[i]
    dists = exact * np.float32(1.01) + rng.normal(0, 0.05, 10).astype(np.float32)
    gt = ids[:7]
    au = runio.AccuracyAudit()
    au.add(ids, dists, q, base, gt)
    sm = au.summary()
    rel = [abs(float(d) - float(e)) / float(e) for d, e in zip(dists, exact)]
    assert math.isclose(sm["mean_relative_error"], sum(rel) / 10, rel_tol=0, abs_tol=1e-15)
    assert sm["p95_relative_error"] == sorted(rel)[9]  # ceil(10 * 0.95) = 10
    assert sm["top10_overlap"] == 0.7
    flips = sum((dists[i] <= dists[j]) != (exact[i] <= exact[j]) for i in range(10) for j in range(i + 1, 10))
    assert sm["pairwise_flip_rate_top10"] == flips / 45
    assert runio.recall_hits(ids, gt) == 7
    assert runio.percentile([5.0, 1.0, 3.0, 2.0], 0.5) == 3.0  # round(1.5) = 2, half away from zero


def _run_and_results():
    run = dict(dataset="toy", method="Ours", status="done", graph_build_distance="exrabitq4_symmetric",
               graph_build_mode="built_in_run", graph_build_distance_evaluations=123456, max_degree=64,
               build_beam=400, alpha=1.2, search_beam_width=1, threads=1, seed=20260813,
               graph_build_time_ms=24890.0, build_time_ms=33910.0, index_size_mb=2850.0, index_bytes=2850000000,
               log_path="x.log", note='gpu "GB300"')
    results = [dict(search_list_size=L, query_coarse_codec="int8", recall=0.9 + L / 1e4, qps=1e5 + L,
                    latency_mean_us=10.5, latency_p95_us=20.25, visited_nodes=1234.5, distance_calls=300.0,
                    mean_relative_error=0.01, p95_relative_error=0.03, mean_absolute_error=0.001,
                    top10_overlap=0.95, pairwise_flip_rate_top10=0.02) for L in (100, 200, 200)]
    return run, results


def test_raw_csv_rows(tmp_path):
    run, results = _run_and_results()
    path = tmp_path / "02_diskann_fair" / "toy" / "csv" / "diskann_fair_raw.csv"
    runio.append_raw_csv(path, run, results)
    runio.append_raw_csv(path, run, results[:1])
    lines = path.read_text().splitlines()
    assert lines[0] == runio.RAW_CSV_HEADER and len(lines) == 5  # one header
    rows = list(csv.DictReader(open(path)))
    assert len(rows[0]) == len(runio.RAW_CSV_HEADER.split(","))
    r = rows[0]
    assert r["alpha"] == "1.2" and r["recall"] == "0.910000" and r["prepare_us"] == "NaN"
    assert float(r["peak_rss_mb"]) > 0 and r["note"] == 'gpu "GB300"' and r["query_coarse_codec"] == "int8"
    assert r["train_time_ms"] == "" and r["index_bytes"] == "2850000000"
    assert r["graph_build_distance_evaluations"] == "123456" and r["repeat_id"] == "aggregate"
    # another schema in an existing file: a reset line, then the header again
    other = tmp_path / "old.csv"
    other.write_text("a,b\n1,2\n")
    runio.append_raw_csv(other, run, results[:1])
    assert other.read_text().splitlines()[2:4] == ["# schema_reset=02_diskann_fair_real_metrics", runio.RAW_CSV_HEADER]


@pytest.mark.skipif(not os.path.isdir(REF), reason="needs the reference tree")
def test_raw_csv_read_by_reference_adapter(tmp_path):
    fn = _ref_function(f"{REF}/experiments/03_system_fair/adapters/ours_adapter.py", "ours_rows_from_02_csv")
    run, results = _run_and_results()
    runio.append_raw_csv(tmp_path / "02_diskann_fair" / "toy" / "csv" / "diskann_fair_raw.csv", run, results)
    rows = fn("toy", tmp_path, 64)
    assert [r["l_search"] for r in rows] == [100, 200]
    assert rows[1]["recall"] == pytest.approx(0.92) and rows[0]["qps"] == pytest.approx(100100.0)
    assert rows[0]["graph_build_time_ms"] == pytest.approx(24890.0)
