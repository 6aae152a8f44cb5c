"""Reader of the ping files written by rtacx::simulation::FileSink
(include/rtacx/simulation.hpp): a sequence of little-endian records
  char[8] "RTACXPNG", uint32 version (1), uint32 range_count,
  uint32 bearing_count, float32 range_min, float32 range_max,
  float32 bearings[bearing_count], complex64 ping[range_count][bearing_count].
"""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np

MAGIC = b"RTACXPNG"


def read_pings(path) -> list[dict]:
    data = Path(path).read_bytes()
    out, pos = [], 0
    while pos < len(data):
        if data[pos:pos + 8] != MAGIC:
            raise ValueError(f"bad record magic at byte {pos}")
        version, nr, nb = struct.unpack_from("<III", data, pos + 8)
        if version != 1:
            raise ValueError(f"unknown ping record version {version}")
        rmin, rmax = struct.unpack_from("<ff", data, pos + 20)
        pos += 28
        bearings = np.frombuffer(data, dtype="<f4", count=nb, offset=pos)
        pos += 4 * nb
        ping = np.frombuffer(data, dtype="<c8", count=nr * nb, offset=pos).reshape(nr, nb)
        pos += 8 * nr * nb
        out.append(dict(range_min=rmin, range_max=rmax, bearings=bearings.copy(), ping=ping.copy()))
    return out
