"""The device arithmetic of the GPU path (quantization_graph_gb300/csrc/qg_device.cuh), compiled for
the host from the same source and run under a warp emulator (tests/native/warp_emu.h: 32 threads
that meet at every shuffle), against the reference's own outputs in tests/golden: the FP32 restore,
the Int8 / Int4 gate and traversal finishes, the residual interval in the two-kernel and the fused
order, the B1 gate, the B1Main distance, the Full codec's gate and mode-1 distance, and the gate
from the encoded record (rabitq_paper_estimate), for every
query x record of the kernel fixtures. The prepared queries are the reference's (the fixtures hold
them), so nothing here depends on the oracle. This checks the routines' arithmetic and lane
order; the kernels that call them are checked on the GPU by tests/test_gpu_*.py."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from cases import kernel_inputs
from conftest import ROOT, load_golden

NATIVE = os.path.join(ROOT, "tests", "native")
CSRC = os.path.join(ROOT, "quantization_graph_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")

KERNEL_CASES = ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536", "kernels_d128_int4",
                "kernels_d1536_int4"]


def _cuda_include():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")
    return inc if os.path.exists(os.path.join(inc, "cuda_fp16.h")) else None


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    inc = _cuda_include()
    if inc is None:
        pytest.skip("the CUDA headers (cuda_fp16.h) are needed to compile the device header for the host")
    out = str(tmp_path_factory.mktemp("devarith") / "libdevarith.so")
    subprocess.run(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-I", NATIVE,
                    "-I", INCLUDE, "-I", CSRC, "-I", inc, os.path.join(NATIVE, "device_arith_check.cpp"), "-o", out],
                   check=True)
    return C.CDLL(out)


def _p(a):
    return C.c_void_p(a.ctypes.data)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _estimates(out6):
    """[n x 6] floats -> the first 21 bytes of RabitqPaperEstimate per row."""
    n = out6.shape[0]
    rows = np.zeros((n, 24), np.uint8)
    rows[:, :20] = np.ascontiguousarray(out6[:, :5], np.float32).view(np.uint8).reshape(n, 20)
    rows[:, 20] = out6[:, 5].astype(np.uint8)
    return rows[:, :21]


def _code_dim(g):
    return g["rotated_residual"].shape[1]


@pytest.mark.parametrize("name", KERNEL_CASES)
def test_int_codec_routines(lib, name):
    """restore_distance_hw (mode 0), finish_gate, finish_traversal (mode 2) and
    residual_interval_thread against the reference, Int8 and Int4 prepared queries."""
    g = load_golden(name)
    D, n, nq = _code_dim(g), int(g["n"]), int(g["nq"])
    rec, msb, fac, res = (np.ascontiguousarray(g[k]) for k in ("compact", "msb", "factors", "residual"))
    for q in range(nq):
        rr = np.ascontiguousarray(g["rotated_residual"][q])
        codes = np.ascontiguousarray(g["codes"][q])
        qn2, qn, half, scale = (float(x) for x in g["scalars"][q])
        csum = int(g["code_sum"][q])
        d0 = np.zeros(n, np.float32)
        assert lib.emu_restore(D, _p(rec), C.c_size_t(rec.shape[1]), C.c_size_t(n), _p(rr), C.c_float(half),
                               C.c_float(qn2), _p(d0)) == 0
        np.testing.assert_array_equal(bits(d0), bits(g["dist_mode0"][q]))
        est = np.zeros((n, 6), np.float32)
        lib.emu_int_gate(D, _p(msb), C.c_size_t(msb.shape[1]), _p(fac), C.c_size_t(fac.shape[1]), C.c_size_t(n),
                         _p(codes), C.c_float(qn2), C.c_float(qn), C.c_float(scale), C.c_longlong(csum),
                         C.c_float(1.9), _p(est))
        np.testing.assert_array_equal(_estimates(est), g["gate"][q][:, :21])
        sip = np.ascontiguousarray(est[:, 1])
        d2 = np.zeros(n, np.float32)
        lib.emu_traversal(D, _p(rec), C.c_size_t(rec.shape[1]), C.c_size_t(n), _p(codes), _p(sip), C.c_float(scale),
                          C.c_longlong(csum), C.c_float(qn2), _p(d2))
        np.testing.assert_array_equal(bits(d2), bits(g["dist_mode2"][q]))
        iv = np.zeros((n, 3), np.float32)
        assert lib.emu_residual(D, _p(res), C.c_size_t(res.shape[1]), C.c_size_t(n), _p(rr), C.c_float(qn), _p(d0),
                                0, _p(iv)) == 0
        np.testing.assert_array_equal(bits(iv), bits(g["residual_iv"][q]))


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_fused_residual_order(lib, name):
    """residual_interval_thread in the fused rerank kernel's product order against
    rabitq_full_residual_distance_batch's outputs."""
    g = load_golden(name)
    v = load_golden("fused_rerank")
    D, n, nq = _code_dim(g), int(g["n"]), int(g["nq"])
    res = np.ascontiguousarray(g["residual"])
    for q in range(nq):
        rr = np.ascontiguousarray(g["rotated_residual"][q])
        d0 = np.ascontiguousarray(g["dist_mode0"][q], np.float32)
        iv = np.zeros((n, 3), np.float32)
        assert lib.emu_residual(D, _p(res), C.c_size_t(res.shape[1]), C.c_size_t(n), _p(rr),
                                C.c_float(float(g["scalars"][q][1])), _p(d0), 1, _p(iv)) == 0
        np.testing.assert_array_equal(bits(iv), bits(v[name][q]))


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d960", "kernels_d1536"])
def test_full_codec_routines(lib, name):
    """full_gate_selected_hw + finish_gate_full (the FP32 gate) and full_distance_hw (mode 1
    with the gate's short ip; mode 0 where reuse is off) against the reference's Full codec."""
    g = load_golden(name)
    v = load_golden("full_codec")
    D, n, nq = _code_dim(g), int(g["n"]), int(g["nq"])
    rec, msb, fac = (np.ascontiguousarray(g[k]) for k in ("compact", "msb", "factors"))
    for q in range(nq):
        rr = np.ascontiguousarray(g["rotated_residual"][q])
        qn2, qn, half, _ = (float(x) for x in g["scalars"][q])
        est = np.zeros((n, 6), np.float32)
        assert lib.emu_full_gate(D, _p(msb), C.c_size_t(msb.shape[1]), _p(fac), C.c_size_t(fac.shape[1]),
                                 C.c_size_t(n), _p(rr), C.c_float(qn2), C.c_float(qn), C.c_float(half), C.c_float(1.9),
                                 _p(est)) == 0
        np.testing.assert_array_equal(_estimates(est), v[f"{name}_gate"][q][:, :21])
        sip = np.ascontiguousarray(est[:, 1])
        reuse = (np.arange(n) % 3 != 0).astype(np.uint8)  # every third record takes mode 0
        d = np.zeros(n, np.float32)
        assert lib.emu_full_distance(D, _p(rec), C.c_size_t(rec.shape[1]), C.c_size_t(n), _p(rr), C.c_float(half),
                                     C.c_float(qn2), _p(reuse), _p(sip), _p(d)) == 0
        want = np.where(reuse == 1, v[f"{name}_dist_mode1"][q], g["dist_mode0"][q]).astype(np.float32)
        np.testing.assert_array_equal(bits(d), bits(want))


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d1536"])
def test_b1_gate_and_b1main_distance(lib, name):
    """finish_gate_b1 with the reference's B1 prepared query, and finish_b1main (the 4-bit x
    +-1 distance) against the reference's query_distance_b1."""
    g = load_golden(name)
    b1 = load_golden("b1_codec")
    b1m = load_golden("b1main_codec")
    D, n, nq = _code_dim(g), int(g["n"]), int(g["nq"])
    rec, msb, fac = (np.ascontiguousarray(g[k]) for k in ("compact", "msb", "factors"))
    _, Q = kernel_inputs(int(g["dim"]), n, nq, int(g["seed"]))
    for q in range(nq):
        qn2, qn = float(g["scalars"][q][0]), float(g["scalars"][q][1])
        ss, es, alpha = (float(x) for x in b1[f"{name}_scalars"][q])
        est = np.zeros((n, 6), np.float32)
        lib.emu_b1_gate(D, _p(msb), C.c_size_t(msb.shape[1]), _p(fac), C.c_size_t(fac.shape[1]), C.c_size_t(n),
                        _p(np.ascontiguousarray(b1[f"{name}_bits"][q])), C.c_float(ss), C.c_float(es),
                        C.c_float(alpha), C.c_float(qn2), C.c_float(qn), C.c_float(1.9), _p(est))
        np.testing.assert_array_equal(_estimates(est), b1[f"{name}_gate"][q][:, :21])
        d = np.zeros(n, np.float32)
        lib.emu_b1main(D, _p(rec), C.c_size_t(rec.shape[1]), C.c_size_t(n),
                       _p(np.ascontiguousarray(g["rotated_residual"][q])), C.c_float(qn2), _p(d))
        np.testing.assert_array_equal(bits(d), bits(b1m[f"{name}_distance_b1"][q]))


@pytest.mark.parametrize("name", ["kernels_d128", "kernels_d100", "kernels_d960", "kernels_d1536"])
def test_encoded_record_gate(lib, name):
    """encoded_short_ip_hw + finish_gate_encoded (compute_paper_prune_estimate) against the
    reference's rabitq_paper_estimate_batch."""
    g = load_golden(name)
    v = load_golden("encoded_gate")
    D, n, nq = _code_dim(g), int(g["n"]), int(g["nq"])
    rec = np.ascontiguousarray(g["compact"])
    for q in range(nq):
        qn2, qn, half, _ = (float(x) for x in g["scalars"][q])
        est = np.zeros((n, 6), np.float32)
        assert lib.emu_encoded_gate(D, _p(rec), C.c_size_t(rec.shape[1]), C.c_size_t(n),
                                    _p(np.ascontiguousarray(g["rotated_residual"][q])), C.c_float(qn2), C.c_float(qn),
                                    C.c_float(half), C.c_float(1.9), _p(est)) == 0
        np.testing.assert_array_equal(_estimates(est), v[f"{name}_c3"][q][:, :21])


def test_invalid_factors_and_degenerate_records(lib, oracle):
    """Rows the fixtures do not hold: sidecar factors whose valid flag is 0 (with finite values)
    and records with zero, negative or NaN norms and zero, NaN or infinite short scales. The
    device routines (Int8 gate, Full gate, encoded-record gate) must refuse exactly where the
    oracle's restatement does and agree with it bit for bit elsewhere."""
    from test_oracle_golden import edge_gate_inputs

    g, rec, fac = edge_gate_inputs()  # the oracle is checked against the reference on the same rows
    D, n = _code_dim(g), int(g["n"])
    _, Q = kernel_inputs(int(g["dim"]), n, int(g["nq"]), int(g["seed"]))
    msb = np.ascontiguousarray(g["msb"])
    ids = np.arange(n, dtype=np.uint32)
    for codec in (3, 0):
        o = oracle.Oracle(int(g["dim"]), g["center"], codec=codec)
        for q in range(2):
            p = o.prepare(Q[q])
            rr = np.ascontiguousarray(p["rotated_residual"])
            qn2, qn, half = float(p["query_norm_sqr"]), float(p["query_norm"]), float(p["half_sum"])
            want = o.gate(ids, msb, fac).view(np.uint8).reshape(n, -1)[:, :21]
            est = np.zeros((n, 6), np.float32)
            if codec == 3:
                lib.emu_int_gate(D, _p(msb), C.c_size_t(msb.shape[1]), _p(fac), C.c_size_t(fac.shape[1]),
                                 C.c_size_t(n), _p(np.ascontiguousarray(p["codes"])), C.c_float(qn2), C.c_float(qn),
                                 C.c_float(float(p["scale"])), C.c_longlong(int(p["code_sum"])), C.c_float(1.9),
                                 _p(est))
            else:
                assert lib.emu_full_gate(D, _p(msb), C.c_size_t(msb.shape[1]), _p(fac), C.c_size_t(fac.shape[1]),
                                         C.c_size_t(n), _p(rr), C.c_float(qn2), C.c_float(qn), C.c_float(half),
                                         C.c_float(1.9), _p(est)) == 0
            np.testing.assert_array_equal(_estimates(est), want)
            assert not want[::3, 20].any()  # the invalid rows were refused
            want_enc = o.gate_encoded(ids, rec).view(np.uint8).reshape(n, -1)[:, :21]
            assert lib.emu_encoded_gate(D, _p(rec), C.c_size_t(rec.shape[1]), C.c_size_t(n), _p(rr), C.c_float(qn2),
                                        C.c_float(qn), C.c_float(half), C.c_float(1.9), _p(est)) == 0
            np.testing.assert_array_equal(_estimates(est), want_enc)
            assert not want_enc[[1, 4, 7, 10, 13, 16], 20].any()
