"""The run_ours driver end to end on a tiny synthetic dataset laid out as the reference's data
directory: the 03 query split, GPU encode, the graph built and saved on the first run and loaded
(unchanged) on the second, an L sweep, and diskann_fair_raw.csv rows in the reference's schema,
one INT8 row per L after the formal-row filter."""
import csv

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_run_ours_writes_rows_and_reuses_its_graph(cuda, oracle, tmp_path):
    from quantization_graph_gb300 import run_ours, runio, synthetic

    # one connected cloud (3,000 points in 64 far-apart clusters would leave the degree-32 graph
    # in pieces that a search from node 0 cannot reach)
    X = synthetic.anisotropic(3000, 128, 0.8, seed=41, normalize=True)
    Q = synthetic.anisotropic(260, 128, 0.8, seed=42, normalize=True)
    gt, _ = oracle.Oracle(128, np.zeros(128, np.float32)).exact_knn(X, Q, 100)
    data = tmp_path / "data" / "tiny"
    data.mkdir(parents=True)
    runio.write_fvecs(data / "tiny_base.fvecs", X)
    runio.write_fvecs(data / "tiny_query.fvecs", Q)
    runio.write_ivecs(data / "tiny_groundtruth.ivecs", gt.astype(np.int32))
    out = tmp_path / "results"
    argv = ["--dataset", "tiny", "--M", "32", "--data-root", str(tmp_path / "data"), "--out-root", str(out),
            "--val-queries", "60", "--search-list-sizes", "20,40,80", "--repeats", "2", "--refine-passes", "1",
            "--build-beam", "100", "--build-batch-size", "256"]
    assert run_ours.main(argv) == 0
    graph = run_ours.graph_path(out, "tiny", 32)
    assert graph.exists()
    first = graph.read_bytes()
    assert run_ours.main(argv) == 0  # the second run loads the frozen graph
    assert graph.read_bytes() == first
    split = out / "03_system_fair" / "tiny" / "csv" / "_query_splits"
    np.testing.assert_array_equal(runio.read_fvecs(split / "test_query.fvecs"), Q[60:])
    path = out / "02_diskann_fair" / "tiny" / "csv" / "diskann_fair_raw.csv"
    with open(path) as f:
        header = f.readline().rstrip("\n")
        rows = list(csv.DictReader([header + "\n"] + [ln for ln in f if not ln.startswith("#")]))
    assert header == runio.RAW_CSV_HEADER
    assert sorted(int(r["search_param_value"]) for r in rows) == [20, 40, 80]  # one formal row per L
    rec = {int(r["search_param_value"]): float(r["recall"]) for r in rows}
    assert rec[20] <= rec[40] <= rec[80] and rec[80] > 0.9, rec
    for r in rows:
        assert r["method"] == "Ours" and r["max_degree"] == "32" and r["query_coarse_codec"] == "int8"
        assert float(r["qps"]) > 0 and float(r["top10_overlap"]) > 0.5
    assert run_ours.log_path(out, "tiny", 32).exists()
