"""Reader (and writer) of the snapshot export container that
nrg_run_export_snapshots writes: the arrays NrgData keeps in its HDF5 file
(nrgData.hpp:134-293), under the same group and dataset names, as a flat
list of named float64 arrays.

Layout: u32 magic 0x4152474e ("NGRA"), u32 version (1), then per array a
u32 name length, the name (UTF-8), a u64 element count and the elements as
little-endian float64.
"""
import struct

import numpy as np

MAGIC = 0x4152474E
VERSION = 1


def read(path):
    """{name: float64 array} of an export file, in file order."""
    with open(path, "rb") as f:
        b = f.read()
    if len(b) < 8:
        raise ValueError("not an NRG export file (too short)")
    magic, ver = struct.unpack_from("<II", b, 0)
    if magic != MAGIC or ver != VERSION:
        raise ValueError("not an NRG export file (magic %#x, version %d)" % (magic, ver))
    out, p = {}, 8
    while p < len(b):
        (n,) = struct.unpack_from("<I", b, p)
        p += 4
        name = b[p:p + n].decode()
        p += n
        (cnt,) = struct.unpack_from("<Q", b, p)
        p += 8
        out[name] = np.frombuffer(b, "<f8", cnt, p).copy()
        p += 8 * cnt
    return out


def write(path, arrays):
    """Write {name: array} in the same container (e.g. the per-iteration
    Eigenvalues<n> an rgflow driver saves beside the snapshots)."""
    with open(path, "wb") as f:
        f.write(struct.pack("<II", MAGIC, VERSION))
        for name, v in arrays.items():
            a = np.ascontiguousarray(v, "<f8").ravel()
            nb = name.encode()
            f.write(struct.pack("<I", len(nb)))
            f.write(nb)
            f.write(struct.pack("<Q", a.size))
            f.write(a.tobytes())


def shell(arrays, iteration):
    """The NrgData view of one saved iteration: sectors, eigenvalues per
    sector, kept counts, coupled indices, eigenvectors (when exported) and
    the operator set as {op: {(row, col): block}}."""
    g = "/NrgItr%d/" % iteration
    nq = int(arrays[g + "nq"][0])
    cur = arrays[g + "current_sysmQ"].astype(int)
    pre = arrays[g + "pre_sysmQ"].astype(int)
    nsec = cur.size // nq if nq else 0
    res = {"current_sysmQ": [tuple(cur[i * nq:(i + 1) * nq]) for i in range(nsec)],
           "pre_sysmQ": [tuple(pre[i * nq:(i + 1) * nq]) for i in range(pre.size // nq if nq else 0)],
           "eigenvaluesQ_kept_indices": arrays[g + "eigenvaluesQ_kept_indices"].astype(int).tolist(),
           "eigenvaluesQ": [arrays[g + "eigenvaluesQ/%d" % s] for s in range(nsec)],
           "coupled_nQ_index": [arrays[g + "coupled_nQ_index/%d" % s].astype(int).tolist() for s in range(nsec)]}
    if g + "current_hamiltonQ/0" in arrays:
        res["current_hamiltonQ"] = []
        for s in range(nsec):
            u = arrays[g + "current_hamiltonQ/%d" % s]
            n = int(round(np.sqrt(u.size)))
            res["current_hamiltonQ"].append(u.reshape(n, n))
    ops = []
    for ip in range(int(arrays[g + "op/operatorSize"][0])):
        og = g + "op/at%d/" % ip
        ids = arrays[og + "idVector"].astype(int).reshape(-1, 2)
        rows, cols = arrays[og + "rowVector"].astype(int), arrays[og + "colVector"].astype(int)
        ops.append({(int(i), int(j)): arrays[og + "qmat%d" % k].reshape(rows[k], cols[k])
                    for k, (i, j) in enumerate(ids)})
    res["ops"] = ops
    return res
