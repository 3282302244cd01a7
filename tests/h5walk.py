"""An independent walk of HDF5 files for the tests, written from the HDF5 File
Format Specification (version 3.0): version 0/1 superblocks, version 1 object
headers, symbol-table groups (v1 B-tree, symbol-table nodes, local heap) and
datasets with compact or contiguous storage of integers, IEEE floats and
fixed-length strings.

Besides returning every dataset ({path: numpy array or str}), it checks the
structural rules a reader relies on and that the library's own reader
enforces: addresses inside the file, the end-of-file address equal to the
file's size, v1 header messages on 8-byte boundaries, B-tree keys that bound
the names of their subtrees (in strcmp order), sorted symbol-table nodes no
fuller than 2K, local-heap free lists inside their data segment, and names
that are NUL-terminated inside their heap.  A violation raises AssertionError.
"""
from __future__ import annotations

import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = (1 << 64) - 1


class Walk:
    def __init__(self, path):
        self.b = open(path, "rb").read()
        off = 0
        while self.b[off:off + 8] != SIG:
            off = 512 if off == 0 else 2 * off
            assert off < len(self.b), "no superblock"
        self.sb = off
        ver = self.b[off + 8]
        assert ver in (0, 1), f"superblock version {ver}"
        assert self.b[off + 13] == 8 and self.b[off + 14] == 8
        self.leafK, self.nodeK = struct.unpack_from("<HH", self.b, off + 16)
        p = off + 24 + (4 if ver == 1 else 0)
        self.base, _free, eof, _drv = struct.unpack_from("<4Q", self.b, p)
        assert eof == len(self.b), f"end-of-file address {eof} != file size {len(self.b)}"
        self.root_entry = p + 32
        _, self.root, cache = struct.unpack_from("<QQI", self.b, self.root_entry)
        self.sets = {}
        self._group(self.root, "", cache_pos=self.root_entry if cache == 1 else None)

    def u(self, fmt, pos):
        assert 0 <= pos and pos + struct.calcsize(fmt) <= len(self.b), "read past the end"
        return struct.unpack_from(fmt, self.b, pos)

    def at(self, rel):
        assert rel != UNDEF and self.base + rel <= len(self.b), "address outside the file"
        return self.base + rel

    def messages(self, rel):
        p = self.at(rel)
        ver, _, nmsg, _ref, size = self.u("<BBHII", p)
        assert ver == 1, "object header version"
        out, chunks = [], [(p + 16, size)]
        while chunks and len(out) < nmsg:
            q, n = chunks.pop(0)
            end = q + n
            while q + 8 <= end and len(out) < nmsg:
                typ, sz, flags = self.u("<HHB", q)
                assert sz % 8 == 0, "v1 message size not a multiple of 8"
                assert q + 8 + sz <= end, "message past its chunk"
                if typ == 0x10:
                    a, ln = self.u("<QQ", q + 8)
                    chunks.append((self.at(a), ln))
                out.append((typ, q + 8, sz, flags))
                q += 8 + sz
        return out

    def heap(self, rel):
        h = self.at(rel)
        assert self.b[h:h + 4] == b"HEAP"
        size, free, seg = self.u("<QQQ", h + 8)
        seg = self.at(seg)
        assert seg + size <= len(self.b)
        # free list inside the segment, terminated by 1
        seen = 0
        while free != 1 and free != UNDEF:
            assert free + 16 <= size, "free block outside the heap"
            nxt, fsz = self.u("<QQ", seg + free)
            assert free + fsz <= size and fsz >= 16
            free = nxt
            seen += 1
            assert seen < 10000
        return seg, size

    def name(self, heap, off):
        seg, size = heap
        assert off < size, "name outside its heap"
        end = self.b.index(b"\0", seg + off)
        assert end < seg + size, "name not terminated inside its heap"
        return self.b[seg + off:end].decode()

    def btree(self, rel, heap, lo, hi, depth=0):
        """Entries of the subtree, checking that its names lie in (lo, hi]."""
        assert depth < 32
        n = self.at(rel)
        assert self.b[n:n + 4] == b"TREE" and self.b[n + 4] == 0
        level, used = self.b[n + 5], self.u("<H", n + 6)[0]
        assert used <= 2 * self.nodeK
        keys = [self.u("<Q", n + 24 + 16 * i)[0] for i in range(used + 1)]
        kids = [self.u("<Q", n + 32 + 16 * i)[0] for i in range(used)]
        names = [self.name(heap, k) for k in keys]
        entries = []
        for i, c in enumerate(kids):
            assert names[i].encode() <= names[i + 1].encode(), "B-tree keys out of order"
            if level > 0:
                entries += self.btree(c, heap, names[i], names[i + 1], depth + 1)
                continue
            s = self.at(c)
            assert self.b[s:s + 4] == b"SNOD" and self.b[s + 4] == 1
            nsym = self.u("<H", s + 6)[0]
            assert 0 < nsym <= 2 * self.leafK
            got = []
            for k in range(nsym):
                e = s + 8 + 40 * k
                noff, oh, cache = self.u("<QQI", e)
                nm = self.name(heap, noff)
                got.append(nm)
                entries.append((nm, oh, cache, e))
            assert [g.encode() for g in got] == sorted(g.encode() for g in got), "unsorted node"
            assert names[i] == "" or names[i].encode() < got[0].encode()
            assert got[-1] == names[i + 1], "key is not the subtree's last name"
        return entries

    def _group(self, rel, path, cache_pos):
        ms = self.messages(rel)
        st = [m for m in ms if m[0] == 0x11]
        assert st, f"group {path or '/'} without a symbol table"
        bt, hp = self.u("<QQ", st[0][1])
        if cache_pos is not None:
            assert self.u("<QQ", cache_pos + 24) == (bt, hp), "stale cached addresses"
        heap = self.heap(hp)
        for nm, oh, cache, epos in self.btree(bt, heap, "", None):
            p = f"{path}/{nm}"
            cms = self.messages(oh)
            types = {m[0] for m in cms}
            if 0x08 in types:
                self.sets[p] = self._dataset(cms)
            elif 0x11 in types:
                self._group(oh, p, epos if cache == 1 else None)

    def _dataset(self, ms):
        m = {t: (pos, sz) for t, pos, sz, _ in ms}
        sp = m[0x01][0]
        ver, rank = self.b[sp], self.b[sp + 1]
        dims = list(self.u("<%dQ" % rank, sp + (8 if ver == 1 else 4))) if rank else []
        tp = m[0x03][0]
        cls, bits = self.b[tp] & 0x0F, self.b[tp + 1]
        size = self.u("<I", tp + 4)[0]
        if cls == 0:
            dt = np.dtype(("<i%d" if bits & 0x08 else "<u%d") % size)
        elif cls == 1:
            dt = np.dtype("<f%d" % size)
        elif cls == 3:
            dt = np.dtype("S%d" % size)
        else:
            raise AssertionError(f"datatype class {cls}")
        lp = m[0x08][0]
        lver = self.b[lp]
        n = int(np.prod(dims)) if dims else 1
        nbytes = n * size
        if lver == 3:
            cls_l = self.b[lp + 1]
            if cls_l == 0:
                raw = self.b[lp + 4:lp + 4 + nbytes]
            else:
                assert cls_l == 1
                a, sz = self.u("<QQ", lp + 2)
                assert sz == nbytes, "contiguous size differs from the dataspace"
                raw = b"\0" * nbytes if a == UNDEF else self.b[self.at(a):self.at(a) + nbytes]
        else:
            assert lver in (1, 2) and self.b[lp + 2] == 1
            a = self.u("<Q", lp + 8)[0]
            raw = self.b[self.at(a):self.at(a) + nbytes]
        assert len(raw) == nbytes
        arr = np.frombuffer(raw, dtype=dt).reshape(dims if dims else ())
        if cls == 3:
            return arr.item().rstrip(b"\0").decode() if not dims else arr
        return arr.copy()


def read(path) -> dict:
    return Walk(path).sets
