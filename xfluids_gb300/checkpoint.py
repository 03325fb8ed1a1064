"""Checkpoint files in the reference's format (XFLUIDS::Output_Ubak / Read_Ubak,
src/XFLUIDS.cpp:658-724): int32 Step, float64 Time, float32 duration, then U (Emax float64 values
per cell, ghost cells included, the reference's AoS layout), packed, little-endian (the byte order
of the x86-64 and aarch64 hosts). The C ABI writes and reads the same files
(xfg_checkpoint_write / xfg_checkpoint_read, xfg_ensemble_checkpoint_write / _add_checkpoint).
"""
from __future__ import annotations

import struct

import numpy as np

HEADER = struct.Struct("<idf")  # 16 bytes, no padding (three sequential writes in the reference)


def write(path, step: int, time: float, duration: float, U: np.ndarray):
    U = np.ascontiguousarray(U, dtype="<f8").reshape(-1)
    with open(path, "wb") as f:
        f.write(HEADER.pack(int(step), float(time), float(duration)))
        f.write(U.tobytes())


def read(path, count: int | None = None):
    """(step, time, duration, U); count = expected number of U values (checked when given)."""
    with open(path, "rb") as f:
        raw = f.read()
    if len(raw) < HEADER.size or (len(raw) - HEADER.size) % 8:
        raise ValueError(f"{path}: not a checkpoint file ({len(raw)} bytes)")
    step, time, duration = HEADER.unpack_from(raw, 0)
    U = np.frombuffer(raw, dtype="<f8", offset=HEADER.size).copy()
    if count is not None and U.size != count:
        raise ValueError(f"{path}: {U.size} values of U, the block needs {count}")
    return step, time, duration, U
