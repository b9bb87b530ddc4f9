"""Reader for the ASTG tensor archives written by the fixture harness (oracle/ref/ref_harness.cpp).

Layout: b"ASTG", u32 count, then per entry: u32 name length, name, u8 dtype
(0 f64, 1 i32, 2 i64, 3 u8), u32 ndim, u64 dims[ndim], raw little-endian data.
"""
import struct

import numpy as np

_DT = {0: np.float64, 1: np.int32, 2: np.int64, 3: np.uint8}


def read(path):
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"ASTG":
        raise ValueError(f"{path}: not an ASTG archive")
    (n,) = struct.unpack_from("<I", buf, 4)
    off = 8
    for _ in range(n):
        (ln,) = struct.unpack_from("<I", buf, off)
        off += 4
        name = buf[off:off + ln].decode()
        off += ln
        dt = _DT[buf[off]]
        off += 1
        (nd,) = struct.unpack_from("<I", buf, off)
        off += 4
        dims = struct.unpack_from("<%dQ" % nd, buf, off)
        off += 8 * nd
        cnt = int(np.prod(dims)) if nd else 1
        nbytes = cnt * np.dtype(dt).itemsize
        out[name] = np.frombuffer(buf, dtype=dt, count=cnt, offset=off).reshape(dims).copy()
        off += nbytes
    return out
