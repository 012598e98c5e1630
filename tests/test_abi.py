"""The C-ABI library builds for sm_103a, loads without a GPU and exports every entry point of
include/qgraph_gb300.h; the product package never reaches the oracle."""
import ctypes
import os
import re
import subprocess

import numpy as np

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "qgraph_gb300.h")


def header_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b((?:rabitq|qg)_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_reference_bridge_symbols():
    names = header_functions()
    assert len([n for n in names if n.startswith("rabitq_")]) == 37


def test_library_builds_and_exports_every_symbol():
    from quantization_graph_gb300 import build

    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (\w+)$", out, flags=re.M))
    missing = [n for n in header_functions() if n not in exported]
    assert not missing, missing
    handle = ctypes.CDLL(lib)  # loads without a GPU (no CUDA call at load time)
    for n in header_functions():
        getattr(handle, n)


def test_python_bindings_cover_the_header():
    from quantization_graph_gb300 import _native

    assert sorted(_native.exported_symbols()) == header_functions()


def test_library_targets_sm103a():
    from quantization_graph_gb300 import build

    assert "arch=compute_103a,code=sm_103a" in build.ARCH


def test_package_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "quantization_graph_gb300")
    for dirpath, _, files in os.walk(pkg):
        if "_build" in dirpath:
            continue
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".h")):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle_py" not in src and "qg_oracle" not in src and "libqg_ref" not in src, f


def test_record_layout_sizes(oracle):
    # space_rabitq.h:2842-2868 with the formal bridge config (external residuals)
    for dim, D, compact, residual, msb in ((128, 128, 81, 88, 16), (960, 1024, 529, 648, 128),
                                           (1024, 1024, 529, 648, 128), (1536, 2048, 1041, 1288, 256)):
        o = oracle.Oracle(dim, np.zeros(dim, np.float32))
        assert (o.D, o.compact_bytes, o.residual_bytes, o.msb_bytes) == (D, compact, residual, msb)


def test_mlp_layout_constants_agree():
    import mlp_ref
    from quantization_graph_gb300 import _native

    text = open(HEADER).read()
    m = re.search(r"#define QG_MLP_PARAMS (\d+)", text)
    assert int(m.group(1)) == mlp_ref.PARAMS == _native.MLP_PARAMS == 4801
    m = re.search(r"#define QG_NOALLOC_SCRATCH_BYTES \(\(size_t\)(\d+) << (\d+)\)", text)
    assert int(m.group(1)) << int(m.group(2)) == _native.QG_NOALLOC_SCRATCH_BYTES


def test_train_centroids_matches_reference(oracle):
    """rabitq_train_centroids (host k-means, rabitq_bridge.cpp:101-172) needs no GPU: called on the
    CPU and compared bit for bit with the reference library's (where it is built)."""
    import ctypes as C

    from quantization_graph_gb300 import build

    if not oracle.reference_available():
        import pytest

        pytest.skip("reference tree not present on this host")
    ours = C.CDLL(build.build())
    ref = oracle.Reference(64, np.zeros(64, np.float32)).lib
    for lib in (ours, ref):
        lib.rabitq_train_centroids.restype = C.c_bool
        lib.rabitq_train_centroids.argtypes = [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_size_t,
                                               C.c_uint32, C.c_int, C.c_void_p]
    rng = np.random.default_rng(0)
    for n, d, k in ((2000, 32, 8), (3000, 128, 64), (1500, 960, 4)):
        X = (rng.standard_normal((n, d)) * rng.uniform(0.1, 2, d)).astype(np.float32)
        a = np.zeros((k, d), np.float32)
        b = np.zeros((k, d), np.float32)
        assert ours.rabitq_train_centroids(X.ctypes.data, n, d, k, min(n, 2500), 7, 10, a.ctypes.data)
        assert ref.rabitq_train_centroids(X.ctypes.data, n, d, k, min(n, 2500), 7, 10, b.ctypes.data)
        np.testing.assert_array_equal(a.view(np.uint32), b.view(np.uint32))
    # the reference's argument checks
    assert not ours.rabitq_train_centroids(X.ctypes.data, n, d, 257, 100, 7, 10, a.ctypes.data)
    assert not ours.rabitq_train_centroids(X.ctypes.data, n, d, 4, 0, 7, 10, a.ctypes.data)
