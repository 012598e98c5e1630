"""ExRaBitQ4 space: the host mirror of the Rust `RabitqSpace` wrapper
(experiments/02_diskann_fair/src/ours_diskann.rs:244-460) over this library's C ABI.

The formal configuration is fixed as in the reference runner (ours_diskann.rs:277): one
centroid, 4-bit residuals in blocks of 16, MSE block scales stored as fp16, rotation seed 100,
INT8 query codec. Encoding, sidecar extraction and query preparation run as CUDA kernels on
torch CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _native as N

CODEC_FULL, CODEC_B1, CODEC_INT4, CODEC_INT8, CODEC_B1MAIN = 0, 1, 2, 3, 4


def _ptr(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(t.data_ptr() if t is not None else 0)


def _stream() -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _cuda(t, dtype) -> torch.Tensor:
    t = torch.as_tensor(t)
    if not t.is_cuda:
        t = t.to("cuda")
    return t.to(dtype).contiguous()


def train_global_center(data: torch.Tensor, sample_count: int = 100_000, seed: int = 100) -> torch.Tensor:
    """Global centre of the data (train_global_center_matrix, diskann_runner.rs:1677-1701).

    For N <= sample_count every row is used and the result is bit-identical to the reference
    (f32 sum in row order times the f32 reciprocal of N). For larger N the reference draws the
    sample with Rust's StdRng, which is not reproducible here; a seeded numpy sample of the same
    size, summed in ascending id order, stands in for it.
    """
    lib = N.load()
    data = _cuda(data, torch.float32)
    n, dim = data.shape
    rows = None
    count = n
    if n > sample_count:
        ids = np.sort(np.random.default_rng(seed).choice(n, size=sample_count, replace=False)).astype(np.uint32)
        rows = torch.from_numpy(ids.view(np.int32)).to("cuda")
        count = sample_count
    out = torch.empty(dim, dtype=torch.float32, device="cuda")
    N.check(lib.qg_center_mean(_ptr(data), dim, dim, _ptr(rows), count, _ptr(out), _stream()), "qg_center_mean")
    return out


class RabitqSpace:
    """One ExRaBitQ4 space (RaBitQSpace in the reference, space_rabitq.h:46)."""

    def __init__(self, dim: int, center, seed: int = 100, codec: int = CODEC_INT8):
        self.lib = N.load()
        self.dim = int(dim)
        ptr = self.lib.rabitq_space_new(self.dim, seed, 1, 4, 16, True, True)
        if not ptr:
            raise RuntimeError(f"rabitq_space_new failed: {N.last_error()}")
        self.ptr = C.c_void_p(ptr)
        center = np.ascontiguousarray(torch.as_tensor(center).detach().cpu().numpy(), dtype=np.float32)
        if center.shape != (self.dim,):
            raise ValueError("center must have shape (dim,)")
        if not self.lib.rabitq_space_set_center(self.ptr, center.ctypes.data):
            raise RuntimeError(f"rabitq_space_set_center failed: {N.last_error()}")
        self.center = center
        self.seed = int(seed)
        self.codec = int(codec)
        self.lib.rabitq_set_query_coarse_codec(self.ptr, codec)
        self.code_dim = self.lib.rabitq_paper_msb_code_bytes(self.ptr) * 8

    def __del__(self):
        try:
            self.lib.rabitq_space_delete(self.ptr)
        except Exception:
            pass

    # record sizes (rabitq_bridge.cpp:174-193, 305-315)
    def full_record_bytes(self) -> int:
        return self.lib.rabitq_full_record_bytes(self.ptr)

    def compact_record_bytes(self) -> int:
        return self.lib.rabitq_compact_record_bytes(self.ptr)

    def residual_record_bytes(self) -> int:
        return self.lib.rabitq_residual_record_bytes(self.ptr)

    def paper_msb_code_bytes(self) -> int:
        return self.lib.rabitq_paper_msb_code_bytes(self.ptr)

    def paper_factor_bytes(self) -> int:
        return self.lib.rabitq_paper_factor_bytes()

    def set_query_coarse_codec(self, codec: int) -> None:
        self.codec = int(codec)
        self.lib.rabitq_set_query_coarse_codec(self.ptr, codec)

    def encode(self, data: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """GPU encode of [n, dim] rows into (compact [n, compact_bytes], residual [n, residual_bytes])
        uint8 CUDA tensors in the reference layouts (encode_ours_payloads, ours_diskann.rs:2150-2203)."""
        data = _cuda(data, torch.float32)
        n = data.shape[0]
        compact = torch.empty((n, self.compact_record_bytes()), dtype=torch.uint8, device="cuda")
        residual = torch.empty((n, self.residual_record_bytes()), dtype=torch.uint8, device="cuda")
        N.check(self.lib.qg_encode_batch(self.ptr, _ptr(data), n, _ptr(compact), _ptr(residual), _stream()),
                "qg_encode_batch")
        return compact, residual

    def encode_gemm(self, data: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """encode() with the rotation as a BF16x3 GEMM on the tensor cores (qg_encode_batch_gemm):
        same layouts; codes equal the reference's except where the GEMM's FP32 summation order
        moves a rotated value across a code boundary."""
        data = _cuda(data, torch.float32)
        n = data.shape[0]
        compact = torch.empty((n, self.compact_record_bytes()), dtype=torch.uint8, device="cuda")
        residual = torch.empty((n, self.residual_record_bytes()), dtype=torch.uint8, device="cuda")
        N.check(self.lib.qg_encode_batch_gemm(self.ptr, _ptr(data), n, _ptr(compact), _ptr(residual), _stream()),
                "qg_encode_batch_gemm")
        return compact, residual

    def rotate_gemm(self, data: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """The encode rotation on the tensor cores (qg_rotate_gemm): ([n, code_dim] rotated
        normalised residuals, [n] residual norms)."""
        data = _cuda(data, torch.float32)
        n = data.shape[0]
        rot = torch.empty((n, self.code_dim), dtype=torch.float32, device="cuda")
        norms = torch.empty(n, dtype=torch.float32, device="cuda")
        N.check(self.lib.qg_rotate_gemm(self.ptr, _ptr(data), n, _ptr(rot), _ptr(norms), _stream()),
                "qg_rotate_gemm")
        return rot, norms

    def signs(self) -> np.ndarray:
        """The rotation's random signs, +-1/sqrt(code_dim) (setRandomRotation, space_rabitq.h:2900-2912)."""
        out = np.empty(self.code_dim, np.float32)
        if not self.lib.qg_space_signs(self.ptr, out.ctypes.data):
            raise RuntimeError(f"qg_space_signs failed: {N.last_error()}")
        return out

    def export_paper_sidecar(self, compact: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
        """MSB plane + 20-byte prune factors per record (rabitq_export_paper_sidecar,
        rabitq_bridge.cpp:317-343), on the GPU."""
        compact = _cuda(compact, torch.uint8)
        n = compact.shape[0]
        msb = torch.empty((n, self.paper_msb_code_bytes()), dtype=torch.uint8, device="cuda")
        factors = torch.empty((n, 20), dtype=torch.uint8, device="cuda")
        N.check(self.lib.qg_export_sidecar_device(self.ptr, _ptr(compact), n, compact.shape[1], _ptr(msb),
                                                  _ptr(factors), _stream()), "qg_export_sidecar_device")
        return msb, factors

    def prepare(self, queries: torch.Tensor) -> dict:
        """Batched query preparation by the space's codec (prepare_query, space_rabitq.h:3700):
        INT8 / INT4 codes, B1 sign bits, B1Main +-1 bytes; the Full codec writes no codes (only
        the rotated residual and the scalars)."""
        q = _cuda(queries, torch.float32)
        nq = q.shape[0]
        D = self.code_dim
        rr = torch.empty((nq, D), dtype=torch.float32, device="cuda")
        codes = torch.empty((nq, D), dtype=torch.int8, device="cuda")
        scal = torch.empty((nq, 4), dtype=torch.float32, device="cuda")
        csum = torch.empty(nq, dtype=torch.int64, device="cuda")
        N.check(self.lib.qg_prepare_batch(self.ptr, _ptr(q), nq, _ptr(rr), _ptr(codes), _ptr(scal), _ptr(csum),
                                          _stream()), "qg_prepare_batch")
        return dict(rotated_residual=rr, codes=codes, scalars=scal, code_sum=csum)

    # kernel-level batched entry points over (query, record) pairs
    def gate_pairs(self, prepared: dict, qidx, ids, msb, factors, epsilon0: float = 1.9) -> torch.Tensor:
        qidx = _cuda(qidx, torch.int32)
        ids = _cuda(ids, torch.int32)
        n = ids.shape[0]
        out = torch.empty((n, 24), dtype=torch.uint8, device="cuda")
        if self.codec not in (CODEC_B1, CODEC_INT4, CODEC_INT8):  # the Full gate (Full, B1Main, variants)
            N.check(self.lib.qg_gate_full_pairs(self.ptr, _ptr(prepared["rotated_residual"]),
                                                _ptr(prepared["scalars"]), _ptr(qidx), _ptr(ids), n, _ptr(msb),
                                                msb.shape[1], _ptr(factors), factors.shape[1], epsilon0, _ptr(out),
                                                _stream()), "qg_gate_full_pairs")
            return out
        N.check(self.lib.qg_gate_pairs(self.ptr, _ptr(prepared["codes"]), _ptr(prepared["scalars"]),
                                       _ptr(prepared["code_sum"]), _ptr(qidx), _ptr(ids), n, _ptr(msb),
                                       msb.shape[1], _ptr(factors), factors.shape[1], epsilon0, _ptr(out),
                                       _stream()), "qg_gate_pairs")
        return out

    def distance_pairs(self, prepared: dict, qidx, ids, modes, records, short_ips) -> torch.Tensor:
        qidx = _cuda(qidx, torch.int32)
        ids = _cuda(ids, torch.int32)
        modes = _cuda(modes, torch.uint8)
        short_ips = _cuda(short_ips, torch.float32)
        n = ids.shape[0]
        out = torch.empty(n, dtype=torch.float32, device="cuda")
        N.check(self.lib.qg_distance_pairs(self.ptr, _ptr(prepared["rotated_residual"]), _ptr(prepared["codes"]),
                                           _ptr(prepared["scalars"]), _ptr(prepared["code_sum"]), _ptr(qidx),
                                           _ptr(ids), _ptr(modes), n, _ptr(records), records.shape[1],
                                           _ptr(short_ips), _ptr(out), _stream()), "qg_distance_pairs")
        return out

    def residual_pairs(self, prepared: dict, qidx, ids, residual, long_distances) -> torch.Tensor:
        qidx = _cuda(qidx, torch.int32)
        ids = _cuda(ids, torch.int32)
        long_distances = _cuda(long_distances, torch.float32)
        n = ids.shape[0]
        out = torch.empty((n, 3), dtype=torch.float32, device="cuda")
        N.check(self.lib.qg_residual_pairs(self.ptr, _ptr(prepared["rotated_residual"]), _ptr(prepared["scalars"]),
                                           _ptr(qidx), _ptr(ids), n, _ptr(residual), residual.shape[1],
                                           _ptr(long_distances), _ptr(out), _stream()), "qg_residual_pairs")
        return out
