"""Minimal read-only HDF5 walker for the golden fixtures.

Only what the reference's HDF5 writer produces is supported: superblock
version 0, symbol-table (v1 B-tree + local heap) groups, version-1 object
headers, and contiguous 1-D datasets of little-endian float64.  It exists
because no HDF5 library is installed here; it is test infrastructure and is
used only by ``make_golden.py``.
"""
import struct

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"


class H5Mini:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        if b[:8] != _SIG:
            raise ValueError("not an HDF5 file: %s" % path)
        if b[8] != 0:
            raise ValueError("only superblock version 0 is supported")
        self.so, self.sl = b[13], b[14]
        if (self.so, self.sl) != (8, 8):
            raise ValueError("only 8-byte offsets/lengths supported")
        # 24 bytes of versions/sizes/K/flags, then 4 addresses, then root entry
        root_entry = 24 + 4 * 8
        _, root_ohdr = struct.unpack_from("<QQ", b, root_entry)
        self.datasets = {}
        self._walk_group(root_ohdr, "")

    # -- object headers -------------------------------------------------
    def _messages(self, addr):
        b = self.b
        ver, _, nmsg, _, hsize = struct.unpack_from("<BBHII", b, addr)
        if ver != 1:
            raise ValueError("only v1 object headers supported")
        blocks = [(addr + 16, hsize)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p < start + size and len(out) < nmsg:
                mtype, msize, _flags = struct.unpack_from("<HHB", b, p)
                data = b[p + 8:p + 8 + msize]
                if mtype == 0x10:  # continuation
                    caddr, clen = struct.unpack_from("<QQ", data, 0)
                    blocks.append((caddr, clen))
                out.append((mtype, data))
                p += 8 + msize
        return out

    def _walk_group(self, ohdr, prefix):
        msgs = self._messages(ohdr)
        stab = [d for t, d in msgs if t == 0x11]
        if not stab:
            return
        btree, heap = struct.unpack_from("<QQ", stab[0], 0)
        heap_data = self._heap_data(heap)
        for name_off, child in self._btree_entries(btree):
            end = self.b.index(b"\0", heap_data + name_off)
            name = self.b[heap_data + name_off:end].decode()
            full = prefix + "/" + name
            cm = self._messages(child)
            types = [t for t, _ in cm]
            if 0x11 in types:
                self._walk_group(child, full)
            elif 0x08 in types:
                self.datasets[full.lstrip("/")] = child

    def _heap_data(self, addr):
        if self.b[addr:addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        return struct.unpack_from("<Q", self.b, addr + 24)[0]

    def _btree_entries(self, addr):
        b = self.b
        if b[addr:addr + 4] != b"TREE":
            raise ValueError("bad B-tree node")
        _ntype, level, used = struct.unpack_from("<BBH", b, addr + 4)
        p = addr + 8 + 16 + 8  # header, siblings, key0
        out = []
        for _ in range(used):
            child = struct.unpack_from("<Q", b, p)[0]
            p += 16  # child + next key
            if level > 0:
                out.extend(self._btree_entries(child))
            else:
                out.extend(self._snod_entries(child))
        return out

    def _snod_entries(self, addr):
        b = self.b
        if b[addr:addr + 4] != b"SNOD":
            raise ValueError("bad symbol node")
        nsym = struct.unpack_from("<H", b, addr + 6)[0]
        out = []
        for k in range(nsym):
            e = addr + 8 + 40 * k
            name_off, ohdr = struct.unpack_from("<QQ", b, e)
            out.append((name_off, ohdr))
        return out

    # -- datasets ---------------------------------------------------------
    def read(self, name):
        msgs = dict((t, d) for t, d in self._messages(self.datasets[name]))
        sp = msgs[0x01]
        ver, ndim = sp[0], sp[1]
        off = 8 if ver == 1 else 4
        dims = struct.unpack_from("<%dQ" % ndim, sp, off)
        dt = msgs[0x03]
        if (dt[0] & 0x0F) != 1 or struct.unpack_from("<I", dt, 4)[0] != 8:
            raise ValueError("only float64 datasets supported (%s)" % name)
        lay = msgs[0x08]
        count = int(np.prod(dims)) if dims else 0
        if lay[0] == 3:
            if lay[1] != 1:
                raise ValueError("only contiguous layout supported")
            addr, size = struct.unpack_from("<QQ", lay, 2)
        else:
            # layout v1/v2: version, ndim, class, 5 reserved, address
            if lay[2] != 1:
                raise ValueError("only contiguous layout supported")
            addr = struct.unpack_from("<Q", lay, 8)[0]
        if count == 0:
            return np.zeros(0)
        if addr == 0xFFFFFFFFFFFFFFFF:
            return np.zeros(count)  # never written: HDF5 fill value 0
        return np.frombuffer(self.b, dtype="<f8", count=count, offset=addr).copy()
