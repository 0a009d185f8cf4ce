"""Reader for the FGV1 golden-vector container written by oracle/ref_pin/fgv_write.h.

Layout: magic b"FGV1", then records ``uint32 name_len, name, uint32 ndim,
uint64 dims[ndim], float64 data[prod(dims)]`` (little-endian). Files may be gzipped.
"""
import gzip
import struct

import numpy as np


def load(path):
    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"FGV1":
        raise ValueError(f"{path}: not an FGV1 file")
    out = {}
    pos = 4
    while pos < len(buf):
        (nl,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        name = buf[pos:pos + nl].decode()
        pos += nl
        (nd,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        dims = struct.unpack_from("<%dQ" % nd, buf, pos)
        pos += 8 * nd
        n = int(np.prod(dims)) if nd else 1
        arr = np.frombuffer(buf, dtype="<f8", count=n, offset=pos).copy()
        pos += 8 * n
        out[name] = arr.reshape(dims) if nd else float(arr[0])
    return out
