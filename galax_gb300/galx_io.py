"""GALX v1 snapshots (galax-io/src/lib.rs:5-92): b"GALX", u32 version 1, u64 n,
f64 timestamp, then x, y, vx, vy, mass, ax, ay as n little-endian f64 each."""
from __future__ import annotations

import struct
import time

import numpy as np

from . import Bodies

MAGIC = b"GALX"
VERSION = 1


class SnapshotError(ValueError):
    pass


def write_snapshot(f, b: Bodies, timestamp: float | None = None) -> None:
    n = len(b)
    f.write(MAGIC)
    f.write(struct.pack("<IQd", VERSION, n, time.time() if timestamp is None else timestamp))
    for a in (b.x, b.y, b.vx, b.vy, b.mass, b.ax, b.ay):
        f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def read_snapshot(f) -> Bodies:
    magic = f.read(4)
    if magic != MAGIC:
        raise SnapshotError("Invalid magic bytes (not a galax snapshot)")
    hdr = f.read(20)
    if len(hdr) < 20:
        raise SnapshotError("Unexpected end of file")
    version, n, _ts = struct.unpack("<IQd", hdr)
    if version != VERSION:
        raise SnapshotError(f"Unsupported version: {version}")
    arrs = []
    for _ in range(7):
        raw = f.read(8 * n)
        if len(raw) < 8 * n:
            raise SnapshotError("Unexpected end of file")
        arrs.append(np.frombuffer(raw, dtype="<f8").astype(np.float64))
    return Bodies(*arrs)
