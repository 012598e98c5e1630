"""fastQuantizeAbs's search over the rescale factor t (space_rabitq.h:867-942), as the encoder runs
it: the warp-parallel form and the one-lane form (quantization_graph_gb300/csrc/code_search.cuh,
compiled for the host unchanged and run under the warp emulator) against the reference's own
algorithm with its min-heap (restated in tests/native/code_search_check.cpp). Every vector must
give the same t bit for bit three ways; the warp form may decline a vector (when its double sums
would not be exact), and then the one-lane form stands."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

NATIVE = os.path.join(ROOT, "tests", "native")
CSRC = os.path.join(ROOT, "quantization_graph_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    if not os.path.exists(os.path.join(inc, "cuda_runtime.h")):
        pytest.skip("the CUDA headers are needed to compile the device code for the host")
    out = str(tmp_path_factory.mktemp("codesearch") / "libqcs.so")
    subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I", NATIVE,
                    "-I", INCLUDE, "-I", CSRC, "-I", inc, os.path.join(NATIVE, "code_search_check.cpp"), "-o", out],
                   check=True)
    return C.CDLL(out)


def _run(lib, v):
    v = np.ascontiguousarray(v, np.float32)
    th, tl, tw = C.c_double(), C.c_double(), C.c_double()
    ok = C.c_int()
    rc = lib.qcs_run(len(v), C.c_void_p(v.ctypes.data), C.byref(th), C.byref(tl), C.byref(tw), C.byref(ok))
    return rc, th.value, tl.value, tw.value, ok.value


def _cases():
    rng = np.random.default_rng(2024)
    for D in (2048, 1024, 128, 64):
        for _ in range(12):
            v = rng.standard_normal(D).astype(np.float32)
            yield "gaussian", v / np.linalg.norm(v)
        for _ in range(4):
            yield "quantised", rng.integers(-12, 13, D).astype(np.float32) * np.float32(0.01)
            yield "power_of_two", (2.0 ** rng.integers(-6, 0, D) * rng.choice([-1, 1, 3, -3, 5, 7], D)).astype(np.float32)
            v = rng.standard_normal(D).astype(np.float32)
            v[rng.choice(D, D // 4, replace=False)] = 0
            v[rng.choice(D, 3, replace=False)] = np.float32(1e-9)
            yield "zeros_and_tiny", v
            v = rng.standard_normal(D).astype(np.float32) * np.float32(1e-3)
            v[0] = 1.0
            yield "one_dominant", v
            yield "all_equal", np.full(D, 0.03, np.float32) * rng.choice([-1, 1], D).astype(np.float32)
            v = rng.standard_normal(D).astype(np.float32)
            v[np.abs(v) < 0.5] = np.float32(2e-5)
            yield "near_1e-5", v


def test_warp_and_lane_searches_equal_the_reference_heap(lib):
    seen, declined = {}, {}
    for kind, v in _cases():
        rc, t_heap, t_lane, t_warp, ok = _run(lib, v)
        assert rc == 0
        assert t_lane == t_heap, (kind, t_lane, t_heap)
        if ok:
            assert t_warp == t_heap, (kind, t_warp, t_heap)
        seen[kind] = seen.get(kind, 0) + 1
        declined[kind] = declined.get(kind, 0) + (0 if ok else 1)
    # the warp form runs on ordinary vectors and declines those whose sums would round
    assert declined["gaussian"] <= 2 and declined["quantised"] == 0 and declined["power_of_two"] == 0
    assert declined["zeros_and_tiny"] == seen["zeros_and_tiny"]
