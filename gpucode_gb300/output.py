"""Reader of the binary column output (WrtBin of libdem_gb300): the
quantities of the reference's Tecplot writer (WriteTec.cpp:9-38) -- X Y Z R
VX VY VZ |w| |F| per particle, one zone per output -- at full precision.

Layout: b"DEMCOL01", int32 column count, 8-byte column names; per zone
b"ZONE\\0\\0\\0\\0", float64 time [s], int64 particle count, then every column
as `count` float64 values."""
from __future__ import annotations

import numpy as np


def read_columns(path) -> tuple[list[str], list[dict]]:
    """-> (column names, zones); each zone {"time": t, "n": n, name: array}"""
    raw = np.fromfile(path, dtype=np.uint8)
    buf = raw.tobytes()
    if buf[:8] != b"DEMCOL01":
        raise ValueError(f"{path}: not a column output file")
    ncol = int(np.frombuffer(buf, np.int32, 1, 8)[0])
    names = [buf[12 + 8 * k: 20 + 8 * k].rstrip(b"\0").decode() for k in range(ncol)]
    off = 12 + 8 * ncol
    zones = []
    while off < len(buf):
        if buf[off:off + 4] != b"ZONE":
            raise ValueError(f"{path}: bad zone tag at byte {off}")
        t = float(np.frombuffer(buf, np.float64, 1, off + 8)[0])
        n = int(np.frombuffer(buf, np.int64, 1, off + 16)[0])
        off += 24
        z = {"time": t, "n": n}
        for name in names:
            z[name] = np.frombuffer(buf, np.float64, n, off).copy()
            off += 8 * n
        zones.append(z)
    return names, zones
