"""DiskANN `.graph.bin` reader/writer (baselines/diskann/diskann-providers/src/storage/bin.rs:234-380).

Layout, little endian: u64 file size, u32 max degree, u32 start id, u64 number of extra
(frozen) start points, then for every node a u32 neighbour count followed by that many u32
ids. The Ours runner appends one frozen start point, whose adjacency is [0]
(ours_diskann.rs:2144-2146), and searches from node 0.
"""
from __future__ import annotations

import numpy as np


def save_graph(path: str, degrees: np.ndarray, edges: np.ndarray, start: int = 0,
               frozen_points: int = 1, max_degree: int | None = None) -> int:
    """Write nodes 0..n-1 from (degrees, edges) plus `frozen_points` frozen start points with
    adjacency [0]; returns the file size."""
    degrees = np.asarray(degrees, dtype=np.uint32)
    edges = np.asarray(edges, dtype=np.uint32)
    n = degrees.shape[0]
    parts = []
    size = 24
    for i in range(n):
        d = int(degrees[i])
        parts.append(np.array([d], np.uint32).tobytes())
        parts.append(edges[i, :d].astype(np.uint32).tobytes())
        size += 4 * (1 + d)
    for _ in range(frozen_points):
        parts.append(np.array([1, 0], np.uint32).tobytes())
        size += 8
    md = int(max_degree if max_degree is not None else max(int(degrees.max(initial=0)), 1))
    header = (np.array([size], np.uint64).tobytes() + np.array([md, start], np.uint32).tobytes()
              + np.array([frozen_points], np.uint64).tobytes())
    with open(path, "wb") as f:
        f.write(header)
        for p in parts:
            f.write(p)
    return size


def load_graph(path: str):
    """Read a graph file; returns (degrees [total], edges [total, max_degree] padded with 0,
    max_degree, start, frozen_points)."""
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size < 24:
        raise ValueError("graph file shorter than its 24-byte header")
    file_size = int(raw[:8].view(np.uint64)[0])
    max_degree, start = (int(v) for v in raw[8:16].view(np.uint32))
    frozen = int(raw[16:24].view(np.uint64)[0])
    if file_size != raw.size:
        raise ValueError(f"graph header size {file_size} != file size {raw.size}")
    words = raw[24:].view(np.uint32)
    degrees = []
    offsets = []
    pos = 0
    while pos < words.size:
        d = int(words[pos])
        if pos + 1 + d > words.size:
            raise ValueError("truncated adjacency list")
        degrees.append(d)
        offsets.append(pos + 1)
        pos += 1 + d
    total = len(degrees)
    width = max(max_degree, max(degrees, default=0), 1)
    edges = np.zeros((total, width), np.uint32)
    for i, (d, o) in enumerate(zip(degrees, offsets)):
        edges[i, :d] = words[o:o + d]
    return np.asarray(degrees, np.uint32), edges, max_degree, start, frozen
