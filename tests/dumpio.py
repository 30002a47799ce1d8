"""Reader for the tagged binary state dumps written by oracle/statedump.h."""
from __future__ import annotations

import struct

import numpy as np

_DT = {"d": np.float64, "i": np.int32, "b": np.uint8, "q": np.int64}


def read_dump(path: str) -> dict[str, np.ndarray]:
    out: dict[str, np.ndarray] = {}
    with open(path, "rb") as fh:
        buf = fh.read()
    if buf[:6] != b"LBDMP1":
        raise ValueError(f"{path}: not a state dump")
    off = 8
    while True:
        (nl,) = struct.unpack_from("<I", buf, off)
        off += 4
        if nl == 0:
            break
        name = buf[off:off + nl].decode()
        off += nl
        dt = chr(buf[off])
        off += 1
        (nd,) = struct.unpack_from("<I", buf, off)
        off += 4
        shape = struct.unpack_from("<%dQ" % nd, buf, off)
        off += 8 * nd
        dtype = np.dtype(_DT[dt])
        count = int(np.prod(shape)) if nd else 1
        arr = np.frombuffer(buf, dtype=dtype, count=count, offset=off).reshape(shape)
        off += count * dtype.itemsize
        out[name] = arr.copy()
    return out
