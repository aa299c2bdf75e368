"""Reader for the named-array files written by oracle/drivers/ref_nrg.cpp
(test infrastructure only)."""
import struct

import numpy as np


def read_named_arrays(path):
    out = {}
    with open(path, "rb") as f:
        b = f.read()
    p = 0
    while p < len(b):
        e = b.index(b"\0", p)
        name = b[p:e].decode()
        p = e + 1
        n = struct.unpack_from("<Q", b, p)[0]
        p += 8
        out[name] = np.frombuffer(b, "<f8", n, p).copy()
        p += 8 * n
    return out
