"""The reference's ExRaBitQ space state file, "EXRBTQ31" (RaBitQSpace::saveState / loadState,
Ours/core/hnswlib/space_rabitq.h:3139-3345), for the formal configuration (one centroid, 4-bit
residuals in blocks of 16, MSE scales stored as fp16, external residual records).

The layout is the reference's, field for field (it is the file format the reference reads):
the 8-byte magic, then little-endian, unpadded

    dim u64, code_dim u64, total_bits u32 (4), short_bits u32 (1), remaining_bits u32 (3),
    header bytes u64 (8), short factor bytes u64 (8), residual factor bytes u64 (8),
    residual scale bytes u64 (D/8), residual bits u32 (4), code bytes u64 (D/2),
    residual code bytes u64 (D/2), compact record bytes u64, compact + residual record bytes u64,
    residual record bytes u64, external residual storage u8 (1), block size u64 (16),
    flags u32 (enabled | block scaling | mse | fp16 = 15), centroid count u64 (1),
    rotation seed u32, centroid f32[dim], rotation signs f32[code_dim].

A space saved here loads in the reference, and a state the reference saved loads here (its
signs replace the ones the seed would generate, as the reference's loader does).
"""
from __future__ import annotations

import struct

import numpy as np

MAGIC = b"EXRBTQ31"
_FIELDS = "<QQIIIQQQQIQQQQQBQIQ"  # the header after the magic, 125 bytes
_FLAGS = 1 | 2 | 4 | 8


def _code_dim(dim: int) -> int:
    rounded = (dim + 63) // 64 * 64  # next_pow2(roundup64(dim)), space_rabitq.h:217-224
    p = 1
    while p < rounded:
        p <<= 1
    return p


def _header(dim: int) -> tuple:
    D = _code_dim(dim)
    compact = 8 + 8 + D // 2 + 1
    residual = 8 + D // 8 + D // 2
    return (dim, D, 4, 1, 3, 8, 8, 8, D // 8, 4, D // 2, D // 2, compact, compact + residual, residual, 1, 16,
            _FLAGS, 1)


def state_bytes(dim: int, seed: int, center, signs) -> bytes:
    """The state as RaBitQSpace::saveState writes it."""
    D = _code_dim(dim)
    center = np.ascontiguousarray(center, dtype="<f4")
    signs = np.ascontiguousarray(signs, dtype="<f4")
    if center.shape != (dim,) or signs.shape != (D,):
        raise ValueError(f"centre must have {dim} floats and signs {D}")
    return MAGIC + struct.pack(_FIELDS, *_header(dim)) + struct.pack("<I", seed) + center.tobytes() + signs.tobytes()


def parse_state(buf: bytes) -> dict:
    """Fields of a state; raises ValueError for another format or configuration, as the
    reference's loader refuses them (space_rabitq.h:3290-3303)."""
    if len(buf) < 8 or buf[:8] != MAGIC:
        raise ValueError("not an EXRBTQ31 state (other ExRaBitQ layouts are not supported)")
    hsize = struct.calcsize(_FIELDS)
    if len(buf) < 8 + hsize + 4:
        raise ValueError("truncated state header")
    fields = struct.unpack_from(_FIELDS, buf, 8)
    dim = fields[0]
    if fields != _header(dim):
        raise ValueError("state of another configuration (bits, block size, flags, centroids or sizes differ)")
    D = fields[1]
    off = 8 + hsize
    (seed,) = struct.unpack_from("<I", buf, off)
    off += 4
    need = off + 4 * dim + 4 * D
    if len(buf) < need:
        raise ValueError("truncated state payload")
    center = np.frombuffer(buf, dtype="<f4", count=dim, offset=off).astype(np.float32)
    signs = np.frombuffer(buf, dtype="<f4", count=D, offset=off + 4 * dim).astype(np.float32)
    if not np.all(np.isfinite(center)):
        raise ValueError("state centroid has non-finite values")
    return dict(dim=dim, code_dim=D, seed=seed, center=center, signs=signs)


def save_state(space, path: str | None = None) -> bytes:
    """Writes (and returns) the state of a RabitqSpace."""
    from . import _native as N

    lib = N.load()
    signs = np.zeros(space.code_dim, np.float32)
    if not lib.qg_space_signs(space.ptr, signs.ctypes.data):
        raise RuntimeError(f"qg_space_signs failed: {N.last_error()}")
    buf = state_bytes(space.dim, space.seed, space.center, signs)
    if path is not None:
        with open(path, "wb") as f:
            f.write(buf)
    return buf


def load_state(src, codec: int | None = None):
    """A RabitqSpace from a state file path or bytes; the stored signs are used."""
    from . import _native as N
    from .space import CODEC_INT8, RabitqSpace

    buf = src if isinstance(src, (bytes, bytearray)) else open(src, "rb").read()
    st = parse_state(bytes(buf))
    space = RabitqSpace(st["dim"], st["center"], seed=st["seed"], codec=CODEC_INT8 if codec is None else codec)
    if not N.load().qg_space_set_signs(space.ptr, np.ascontiguousarray(st["signs"]).ctypes.data):
        raise RuntimeError(f"qg_space_set_signs failed: {N.last_error()}")
    return space
