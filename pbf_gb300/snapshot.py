"""The binary state snapshot format of pbf_save_state / pbf_load_state, read
and written on the host without a device handle.

Layout (little-endian): the 8 bytes "PBFSTATE", u32 format version (1),
u32 particle count n, u32 scene count, u32 0, then positions and velocities
as float4[n] each, in particle-id order (w lanes as stored).  The reference
has no snapshot; it only resets to its initial blocks
(src/Simulation.cpp:303-305).
"""
from __future__ import annotations

import numpy as np

MAGIC = b"PBFSTATE"
VERSION = 1
HEADER_BYTES = 24


def write_snapshot(path, x4, v4, num_scenes: int = 1) -> None:
    x = np.ascontiguousarray(x4, np.float32)
    v = np.ascontiguousarray(v4, np.float32)
    if x.ndim != 2 or x.shape[1] != 4 or v.shape != x.shape:
        raise ValueError("x4 and v4 must be float32 arrays of shape (n, 4)")
    hdr = np.array([VERSION, x.shape[0], int(num_scenes), 0], "<u4")
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(hdr.tobytes())
        f.write(x.astype("<f4").tobytes())
        f.write(v.astype("<f4").tobytes())


def read_snapshot(path):
    """Returns (x4, v4, num_scenes)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < HEADER_BYTES or data[:8] != MAGIC:
        raise ValueError(f"{path}: not a state snapshot")
    version, n, scenes, _ = np.frombuffer(data, "<u4", 4, 8)
    if version != VERSION:
        raise ValueError(f"{path}: snapshot version {version}, expected {VERSION}")
    if len(data) != HEADER_BYTES + 32 * int(n):
        raise ValueError(f"{path}: truncated snapshot")
    body = np.frombuffer(data, "<f4", 8 * int(n), HEADER_BYTES).reshape(2, int(n), 4)
    return body[0].astype(np.float32), body[1].astype(np.float32), int(scenes)
