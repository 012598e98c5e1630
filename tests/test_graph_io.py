import numpy as np
import pytest

from conftest import load_golden
from quantization_graph_gb300.graph_io import load_graph, save_graph


def test_roundtrip_with_frozen_start(tmp_path):
    g = load_golden("search_c1")
    p = tmp_path / "g.graph.bin"
    size = save_graph(str(p), g["degrees"], g["edges"], start=123, frozen_points=1, max_degree=32)
    assert size == p.stat().st_size
    deg, edges, md, start, frozen = load_graph(str(p))
    n = len(g["degrees"])
    assert md == 32 and start == 123 and frozen == 1 and len(deg) == n + 1
    np.testing.assert_array_equal(deg[:n], g["degrees"])
    for i in range(0, n, 97):
        np.testing.assert_array_equal(edges[i, :deg[i]], g["edges"][i, :g["degrees"][i]])
    assert deg[n] == 1 and edges[n, 0] == 0


def test_truncated_file_is_rejected(tmp_path):
    p = tmp_path / "bad.graph.bin"
    save_graph(str(p), np.array([2, 1], np.uint32), np.array([[1, 0], [0, 0]], np.uint32))
    raw = p.read_bytes()
    p.write_bytes(raw[:-4])
    with pytest.raises(ValueError):
        load_graph(str(p))
