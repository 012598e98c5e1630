"""The float-float fast path of the symmetric 4-bit estimator (csrc/sym_ff.cuh), compiled for the
host from the same source the GPU build uses, against the double-precision expression of
symmetricBuildDistanceFromPrepared (space_rabitq.h:2706-2747) and against the oracle: whenever
the fast path answers, its float is the double expression's float, bit for bit."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

SRC = os.path.join(ROOT, "tests", "native", "sym_ff_check.cpp")
INC = os.path.join(ROOT, "quantization_graph_gb300", "csrc")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("symff") / "libsymff.so")
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I", INC, SRC, "-o", out],
                   check=True)
    lib = C.CDLL(out)
    lib.sym_ff_compare.restype = C.c_int64
    return lib


def _run(lib, n2l, lsl, n2r, lsr, s):
    arrs = [np.ascontiguousarray(a, dt) for a, dt in ((n2l, np.float32), (lsl, np.float32), (n2r, np.float32),
                                                       (lsr, np.float32), (s, np.int32))]
    n = len(arrs[-1])
    ff = np.zeros(n, np.float32)
    f64 = np.zeros(n, np.float32)
    taken = np.zeros(n, np.uint8)
    p = [C.c_void_p(a.ctypes.data) for a in arrs]
    bad = lib.sym_ff_compare(*p, C.c_size_t(n), C.c_void_p(ff.ctypes.data), C.c_void_p(f64.ctypes.data),
                             C.c_void_p(taken.ctypes.data))
    return bad, ff, f64, taken.astype(bool)


def _records(g):
    c = g["compact"]
    n2 = c[:, 0:4].copy().view(np.float32)[:, 0]
    ls = c[:, 4:8].copy().view(np.float32)[:, 0]
    D = (c.shape[1] - 17) * 2
    codes = c[:, 16:16 + D // 2]
    nib = np.empty((c.shape[0], D), np.int64)
    nib[:, 0::2] = codes & 15
    nib[:, 1::2] = codes >> 4
    return n2, ls, 2 * nib - 15


@pytest.mark.parametrize("name", ["search_c1", "search_c2", "search_c3"])
def test_fast_path_equals_double_on_encoded_records(lib, oracle, name):
    g = load_golden(name)
    n2, ls, cen = _records(g)
    rng = np.random.default_rng(3)
    n = len(n2)
    i = rng.integers(0, n, 200_000)
    j = rng.integers(0, n, 200_000)
    s = np.einsum("ij,ij->i", cen[i], cen[j]).astype(np.int32)
    bad, ff, f64, taken = _run(lib, n2[i], ls[i], n2[j], ls[j], s)
    assert bad == 0
    assert taken.mean() > 0.995, taken.mean()
    # the double expression here is the oracle's symmetric distance
    o = oracle.Oracle(int(g["dim"]), g["center"])
    for k in range(0, 2000, 7):
        ref = o.symmetric_distance(g["compact"][i[k]], g["compact"][j[k]])
        assert np.float32(ref).view(np.uint32) == f64[k].view(np.uint32)


def test_fast_path_on_adversarial_inputs(lib):
    """Near-identical records (heavy cancellation), products at the clamp |u| = 1, zero and
    extreme magnitudes, signed zeros, and random magnitudes over twelve decades."""
    rng = np.random.default_rng(7)
    m = 400_000
    n2l = (10.0 ** rng.uniform(-6, 6, m)).astype(np.float32)
    n2r = np.where(rng.random(m) < 0.3, n2l, (10.0 ** rng.uniform(-6, 6, m))).astype(np.float32)
    lsl = (np.sqrt(n2l) * rng.uniform(1.6, 2.4, m)).astype(np.float32)
    lsr = (np.sqrt(n2r) * rng.uniform(1.6, 2.4, m)).astype(np.float32)
    D = 2048
    # s near the value that makes u = 1: u = s/4 * ls_l/(2 rn_l) * ls_r/(2 rn_r)
    unit = 16.0 * np.sqrt(n2l.astype(np.float64) * n2r) / (lsl.astype(np.float64) * lsr)
    near = np.round(unit * rng.uniform(0.999, 1.001, m))
    s = np.where(rng.random(m) < 0.5, near, rng.integers(-225 * D, 225 * D, m)).clip(-225 * D, 225 * D)
    s[:100] = 0
    lsl[100:200] = 0.0  # invalid lhs
    n2l[200:300] = 0.0
    bad, ff, f64, taken = _run(lib, n2l, lsl, n2r, lsr, s.astype(np.int32))
    assert bad == 0
    assert not taken[100:300].any()  # invalid records always take the double path
    assert taken.mean() > 0.8  # half the pairs sit at the clamp on purpose
