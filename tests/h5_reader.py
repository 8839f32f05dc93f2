"""A strict reader of the HDF5 structures that solution files use — test
infrastructure, written from the HDF5 File Format Specification (The HDF
Group), independently of the library's encoder.

It reads superblock versions 0 and 1, version-1 object headers (with
continuation blocks), groups held in symbol tables (version-1 B-tree of group
nodes, symbol-table nodes, local heap), datatypes of class fixed point,
floating point and string, version-1/2 dataspaces, contiguous and compact
layouts (versions 1-3) and version-1 to 3 attribute messages.  On the way it
checks the invariants an HDF5 library relies on when it opens such a file:
signatures and versions, the end-of-file address against the file's length,
message sizes in multiples of 8 and message counts against the header
prefix, the local heap's free list (terminated by offset 1) inside its data
segment, B-tree keys in increasing name order that bracket each child's
names, symbol-table nodes within their capacity and sorted, the root entry's
cached B-tree and heap addresses against its symbol-table message, data
inside the file.  Anything else raises H5FormatError.
"""
from __future__ import annotations

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5FormatError(Exception):
    pass


def _need(cond, msg):
    if not cond:
        raise H5FormatError(msg)


class Dataset:
    def __init__(self, name, data, attrs, messages):
        self.name = name
        self.data = data
        self.attrs = attrs
        self.messages = messages  # [(type, flags, body bytes)]


class H5File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        b = self.b
        off = 0
        while off < len(b) and b[off:off + 8] != SIGNATURE:
            off = 512 if off == 0 else off * 2
        _need(off < len(b), "no HDF5 signature")
        self.sb = off
        v = b[off + 8]
        _need(v in (0, 1), f"superblock version {v} not read here")
        _need(b[off + 9] == 0 and b[off + 10] == 0 and b[off + 12] == 0, "superblock sub-versions")
        _need(b[off + 13] == 8 and b[off + 14] == 8, "sizes of offsets/lengths must be 8")
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", b, off + 16)
        _need(self.leaf_k > 0 and self.internal_k > 0, "group K values")
        p = off + 24
        if v == 1:
            p += 4  # indexed storage internal node K + reserved
        base, free_addr, eof, drv = struct.unpack_from("<QQQQ", b, p)
        self.base = base
        _need(base == off, "base address must be the superblock's offset")
        _need(eof == len(b), f"end-of-file address {eof} != file length {len(b)}")
        _need(free_addr == UNDEF, "free-space info not expected")
        self.root_entry = self._entry(p + 32)
        name_off, oh, cache, scratch = self.root_entry
        self.root_messages = self._object_header(oh)
        stab = [m for m in self.root_messages if m[0] == 0x11]
        _need(len(stab) == 1, "root group needs one symbol-table message")
        tree, heap = struct.unpack_from("<QQ", stab[0][2])
        if cache == 1:
            _need(struct.unpack_from("<QQ", scratch) == (tree, heap),
                  "root entry's cached B-tree/heap addresses differ from its symbol table")
        self.heap = self._local_heap(heap)
        self.entries = self._group(tree)  # [(name, object header address)] in order
        self.names = [n for n, _ in self.entries]
        self.attrs = self._attributes(self.root_messages)
        self.datasets = {}
        for name, addr in self.entries:
            msgs = self._object_header(addr)
            self.datasets[name] = Dataset(name, self._data(msgs), self._attributes(msgs), msgs)

    # ---- primitives --------------------------------------------------------
    def _at(self, addr, n):
        a = self.base + addr
        _need(addr != UNDEF and 0 <= a and a + n <= len(self.b), f"address {addr:#x}+{n} outside")
        return self.b[a:a + n]

    def _entry(self, pos):
        name_off, oh, cache, _res = struct.unpack_from("<QQII", self.b, pos)
        _need(cache in (0, 1, 2), "symbol-table entry cache type")
        return name_off, oh, cache, self.b[pos + 24:pos + 40]

    def _object_header(self, addr):
        pre = self._at(addr, 16)
        ver, res, nmsg, refc, size = struct.unpack_from("<BBHII", pre)
        _need(ver == 1 and res == 0, f"object header version {ver}")
        _need(refc >= 1, "object reference count")
        msgs = []
        chunks = [(addr + 16, size)]
        while chunks:
            a, n = chunks.pop(0)
            body = self._at(a, n)
            p = 0
            while p < n:
                _need(p + 8 <= n, "message header past the chunk")
                mtype, msize, flags = struct.unpack_from("<HHB", body, p)
                _need(msize % 8 == 0, f"message size {msize} not a multiple of 8")
                _need(p + 8 + msize <= n, "message past the chunk")
                data = body[p + 8:p + 8 + msize]
                msgs.append((mtype, flags, data))
                if mtype == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", data)
                    chunks.append((caddr, clen))
                p += 8 + msize
        _need(len(msgs) == nmsg, f"{len(msgs)} messages found, prefix says {nmsg}")
        return msgs

    def _local_heap(self, addr):
        h = self._at(addr, 32)
        _need(h[:4] == b"HEAP" and h[4] == 0, "local heap signature/version")
        size, free, data_addr = struct.unpack_from("<QQQ", h, 8)
        seg = self._at(data_addr, size)
        seen = set()
        while free != 1:
            _need(free % 8 == 0 and free + 16 <= size and free not in seen, "heap free list")
            seen.add(free)
            nxt, blk = struct.unpack_from("<QQ", seg, free)
            _need(blk >= 16 and free + blk <= size, "heap free block size")
            free = nxt
        _need(seg[:1] == b"\0", "the heap's first name must be the empty string")
        return seg

    def _heap_name(self, off):
        _need(off < len(self.heap), "name offset outside the heap")
        end = self.heap.index(b"\0", off)
        return self.heap[off:end].decode()

    def _group(self, tree):
        h = self._at(tree, 24)
        _need(h[:4] == b"TREE", "B-tree signature")
        ntype, level, used = struct.unpack_from("<BBH", h, 4)
        _need(ntype == 0, "group B-tree expected")
        _need(1 <= used <= 2 * self.internal_k, f"B-tree entries used {used}")
        body = self._at(tree + 24, (2 * used + 1) * 8)
        keys = [struct.unpack_from("<Q", body, 16 * i)[0] for i in range(used + 1)]
        kids = [struct.unpack_from("<Q", body, 16 * i + 8)[0] for i in range(used)]
        knames = [self._heap_name(k) for k in keys]
        for i in range(used):
            _need(knames[i] < knames[i + 1] or (i == 0 and knames[0] == knames[1] == ""),
                  "B-tree keys out of order")
        out = []
        for i, c in enumerate(kids):
            part = self._group(c) if level > 0 else self._snod(c)
            for name, _ in part:
                _need(knames[i] < name <= knames[i + 1],
                      f"name {name!r} outside its B-tree key range")
            out += part
        return out

    def _snod(self, addr):
        h = self._at(addr, 8)
        _need(h[:4] == b"SNOD" and h[4] == 1, "symbol-table node signature/version")
        n = struct.unpack_from("<H", h, 6)[0]
        _need(1 <= n <= 2 * self.leaf_k, f"symbol-table node holds {n}")
        self._at(addr, 8 + 2 * self.leaf_k * 40)  # the node's full size lies inside the file
        out = []
        for k in range(n):
            name_off, oh, cache, _ = self._entry(self.base + addr + 8 + 40 * k)
            out.append((self._heap_name(name_off), oh))
        names = [x for x, _ in out]
        _need(names == sorted(names) and len(set(names)) == n, "symbol-table node not sorted")
        return out

    # ---- messages ----------------------------------------------------------
    @staticmethod
    def _datatype(d):
        cv = d[0]
        ver, cls = cv >> 4, cv & 15
        _need(ver in (1, 2, 3), "datatype version")
        bits = d[1:4]
        size = struct.unpack_from("<I", d, 4)[0]
        if cls == 0:
            _need(len(d) >= 12, "fixed-point properties")
            _need(bits[0] & 1 == 0, "big-endian integers not read here")
            signed = bool(bits[0] & 8)
            return (("<i" if signed else "<u") + str(size)), size, 12
        if cls == 1:
            _need(len(d) >= 20, "floating-point properties")
            _need(bits[0] & 1 == 0, "big-endian floats not read here")
            _, prec, eloc, esize, mloc, msize, bias = struct.unpack_from("<HHBBBBI", d, 8)
            _need((size, prec, eloc, esize, mloc, msize, bias) in
                  ((8, 64, 52, 11, 0, 52, 1023), (4, 32, 23, 8, 0, 23, 127)), "non-IEEE float")
            return "<f" + str(size), size, 20
        if cls == 3:
            _need(bits[0] & 15 in (0, 1, 2) and bits[0] >> 4 in (0, 1), "string padding/charset")
            return ("S", bits[0] & 15), size, 8
        raise H5FormatError(f"datatype class {cls} not read here")

    @staticmethod
    def _dataspace(d):
        ver, rank = d[0], d[1]
        if ver == 1:
            _need(len(d) >= 8 + 8 * rank, "dataspace size")
            return tuple(struct.unpack_from("<%dQ" % rank, d, 8)), 8 + 8 * rank * (
                2 if d[2] & 1 else 1)
        if ver == 2:
            _need(d[3] in (0, 1), "null dataspaces not read here")
            return tuple(struct.unpack_from("<%dQ" % rank, d, 4)), 4 + 8 * rank * (
                2 if d[2] & 1 else 1)
        raise H5FormatError(f"dataspace version {ver}")

    @staticmethod
    def _decode(raw, dtype, shape):
        if isinstance(dtype, tuple):
            s = raw
            if dtype[1] in (0, 1):
                s = s.split(b"\0", 1)[0]
            else:
                s = s.rstrip(b" ")
            return s.decode("utf-8")
        a = np.frombuffer(raw, dtype=dtype).copy()
        return a[0].item() if shape == () else a.reshape(shape)

    def _attributes(self, msgs):
        out = {}
        for mtype, _flags, d in msgs:
            if mtype != 0x0C:
                continue
            ver = d[0]
            nlen, tlen, slen = struct.unpack_from("<HHH", d, 2)
            p = 8 if ver in (1, 2) else 9
            pad = (lambda n: (n + 7) & ~7) if ver == 1 else (lambda n: n)
            name = d[p:p + nlen].split(b"\0", 1)[0].decode()
            p += pad(nlen)
            dtype, esize, _ = self._datatype(d[p:p + tlen])
            p += pad(tlen)
            shape, _ = self._dataspace(d[p:p + slen])
            p += pad(slen)
            count = int(np.prod(shape)) if shape else 1
            raw = d[p:p + esize * count]
            _need(len(raw) == esize * count, f"attribute {name}: data past the message")
            _need(name not in out, f"duplicate attribute {name}")
            out[name] = self._decode(raw, dtype, shape)
        return out

    def _data(self, msgs):
        by = {}
        for mtype, _flags, d in msgs:
            by.setdefault(mtype, []).append(d)
        _need(1 in by and 3 in by and 8 in by, "dataset needs dataspace, datatype, layout")
        shape, _ = self._dataspace(by[1][0])
        dtype, esize, _ = self._datatype(by[3][0])
        lay = by[8][0]
        count = int(np.prod(shape)) if shape else 1
        if lay[0] in (1, 2):
            rank, cls = lay[1], lay[2]
            _need(cls == 1, "only contiguous v1/v2 layouts read here")
            addr = struct.unpack_from("<Q", lay, 8)[0]
            dims = struct.unpack_from("<%dI" % rank, lay, 16)
            _need(dims[-1] == esize, "layout element size")
            nbytes = count * esize
        elif lay[0] == 3:
            cls = lay[1]
            if cls == 0:
                nbytes = struct.unpack_from("<H", lay, 2)[0]
                _need(nbytes == count * esize, "compact data size")
                return self._decode(lay[4:4 + nbytes], dtype, shape)
            _need(cls == 1, "only contiguous and compact v3 layouts read here")
            addr, nbytes = struct.unpack_from("<QQ", lay, 2)
            _need(nbytes == count * esize, "contiguous size != dataspace x element size")
        else:
            raise H5FormatError(f"layout version {lay[0]}")
        if count == 0:
            return np.zeros(shape, dtype=dtype)
        return self._decode(self._at(addr, nbytes), dtype, shape)
