"""Minimal HDF5 reader for the tests (pure Python, from the HDF5 file-format
specification): superblock v0/v1 (with user block), version-1 object headers
with continuation blocks, symbol-table groups (any B-tree depth), version 1-3
attribute messages, contiguous/compact float and integer datasets.  It is an
independent second reader for files written by the library and is also run
on a libhdf5-written file."""
import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        at = 0
        while self.b[at:at + 8] != SIG:
            at = 512 if at == 0 else at * 2
            if at >= len(self.b):
                raise ValueError("no superblock")
        v = self.b[at + 8]
        if v > 1:
            raise ValueError("superblock version %d not handled" % v)
        self.so, self.sl = self.b[at + 13], self.b[at + 14]
        self.leaf_k, self.int_k = struct.unpack_from("<HH", self.b, at + 16)
        p = at + 24 + (4 if v == 1 else 0)
        self.base = self.u(p, self.so) or at
        self.eof = self.u(p + 2 * self.so, self.so)
        p += 4 * self.so
        self.root = self.u(p + self.so, self.so)

    def u(self, p, n):
        return int.from_bytes(self.b[p:p + n], "little")

    def a(self, addr):
        return self.base + addr

    def messages(self, oh):
        p = self.a(oh)
        if self.b[p] != 1:
            raise ValueError("object header version %d" % self.b[p])
        nmsg, _, size = struct.unpack_from("<HII", self.b, p + 2)
        chunks, out, seen = [(p + 16, size)], [], 0
        while chunks and seen < nmsg:
            q, n = chunks.pop(0)
            end = q + n
            while q + 8 <= end and seen < nmsg:
                t, sz = struct.unpack_from("<HH", self.b, q)
                data = self.b[q + 8:q + 8 + sz]
                if t == 0x10:
                    chunks.append((self.a(self.u(q + 8, self.so)), self.u(q + 8 + self.so, self.sl)))
                else:
                    out.append((t, data))
                q += 8 + sz
                seen += 1
        return out

    def links(self, oh):
        res = {}
        for t, d in self.messages(oh):
            if t != 0x11:
                continue
            bt, hp = self.u_(d, 0), self.u_(d, self.so)
            h = self.a(hp)
            assert self.b[h:h + 4] == b"HEAP"
            hsize = self.u(h + 8, self.sl)
            hdata = self.a(self.u(h + 8 + 2 * self.sl, self.so))
            names = self.b[hdata:hdata + hsize]

            def walk(node):
                n = self.a(node)
                assert self.b[n:n + 4] == b"TREE", "bad B-tree node"
                level, used = self.b[n + 5], struct.unpack_from("<H", self.b, n + 6)[0]
                body = n + 8 + 2 * self.so
                for k in range(used):
                    child = self.u(body + self.sl + k * (self.so + self.sl), self.so)
                    if level:
                        walk(child)
                        continue
                    s = self.a(child)
                    assert self.b[s:s + 4] == b"SNOD", "bad symbol table node"
                    ns = struct.unpack_from("<H", self.b, s + 6)[0]
                    esz = 2 * self.so + 24
                    for e in range(ns):
                        q = s + 8 + e * esz
                        off = self.u(q, self.so)
                        name = names[off:names.index(b"\0", off)].decode()
                        res[name] = self.u(q + self.so, self.so)
            walk(bt)
        return res

    def u_(self, d, p, n=None):
        n = n or self.so
        return int.from_bytes(d[p:p + n], "little")

    def resolve(self, path):
        oh = self.root
        for part in [x for x in path.split("/") if x]:
            oh = self.links(oh)[part]
        return oh

    @staticmethod
    def _dtype(dt):
        cls, size = dt[0] & 15, struct.unpack_from("<I", dt, 4)[0]
        if cls == 1:
            return np.dtype("<f8" if size == 8 else "<f4")
        if cls == 0:
            signed = bool(dt[1] & 8)
            return np.dtype(("<i" if signed else "<u") + str(size))
        if cls == 3:
            return np.dtype("S%d" % size)
        raise ValueError("datatype class %d" % cls)

    @staticmethod
    def _dims(ds):
        ver, rank = ds[0], ds[1]
        o = 8 if ver == 1 else 4
        return [int.from_bytes(ds[o + 8 * k:o + 8 * k + 8], "little") for k in range(rank)]

    def attrs(self, path):
        out = {}
        for t, d in self.messages(self.resolve(path)):
            if t != 0x0C:
                continue
            ver = d[0]
            nsz, dtsz, dssz = struct.unpack_from("<HHH", d, 2)
            p = 8 + (1 if ver == 3 else 0)
            al = (lambda n: (n + 7) // 8 * 8) if ver == 1 else (lambda n: n)
            name = d[p:p + nsz - 1].decode()
            p += al(nsz)
            dt = d[p:p + dtsz]
            p += al(dtsz)
            ds = d[p:p + dssz]
            p += al(dssz)
            typ = self._dtype(dt)
            n = int(np.prod(self._dims(ds))) if self._dims(ds) else 1
            val = np.frombuffer(d[p:p + n * typ.itemsize], dtype=typ)
            out[name] = val[0] if n == 1 else val
        return out

    def dataset(self, path):
        dims, typ, addr, compact = None, None, None, None
        for t, d in self.messages(self.resolve(path)):
            if t == 1:
                dims = self._dims(d)
            elif t == 3:
                typ = self._dtype(d)
            elif t == 8:
                if d[0] >= 3 and d[1] == 1:
                    addr = self.u_(d, 2)
                elif d[0] >= 3 and d[1] == 0:
                    compact = d[4:4 + struct.unpack_from("<H", d, 2)[0]]
                elif d[0] < 3 and d[2] == 1:
                    addr = self.u_(d, 8)
                else:
                    raise ValueError("layout not handled")
        n = int(np.prod(dims))
        if compact is not None:
            raw = compact
        elif addr == UNDEF:
            return np.zeros(dims, dtype=typ)
        else:
            raw = self.b[self.a(addr):self.a(addr) + n * typ.itemsize]
        return np.frombuffer(raw, dtype=typ).reshape(dims)
