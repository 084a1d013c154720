"""A small HDF5 reader for the files sledgehamr writes, used by the tests.

sledgehamr's writers (source/utils/hdf5_utils.h:80-104) put one-dimensional
contiguous datasets of IEEE floats into the root group of a file created
with the library's default (earliest) format: a version-0 superblock, a
symbol-table root group (version-1 B-tree of symbol-table nodes plus a local
heap of names) and version-1 object headers.  This reader follows the
published HDF5 file format specification for exactly those structures and
rejects anything else, so it can check both the reference's own data file
(data/spectra_ks.hdf5, written by h5py) and the files the library writes.

Test infrastructure only: the library never imports it.
"""
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class Hdf5Error(Exception):
    pass


def _u(buf, off, n):
    return int.from_bytes(buf[off:off + n], "little")


class Message:
    def __init__(self, mtype, flags, data):
        self.type = mtype
        self.flags = flags
        self.data = data


class Dataset:
    def __init__(self, name, shape, dtype, addr, nbytes, messages):
        self.name = name
        self.shape = shape
        self.dtype = dtype
        self.addr = addr
        self.nbytes = nbytes
        self.messages = messages


class File:
    """Parses the whole file at construction; datasets are read lazily."""

    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        b = self.buf
        if b[:8] != SIGNATURE:
            raise Hdf5Error("no HDF5 signature at offset 0")
        if b[8] != 0:
            raise Hdf5Error("superblock version %d (only 0 is read)" % b[8])
        if b[13] != 8 or b[14] != 8:
            raise Hdf5Error("offsets and lengths must be 8 bytes")
        self.leaf_k = _u(b, 16, 2)
        self.internal_k = _u(b, 18, 2)
        base = _u(b, 24, 8)
        if base != 0:
            raise Hdf5Error("base address %d" % base)
        self.eof = _u(b, 40, 8)
        if self.eof != len(b):
            raise Hdf5Error("end-of-file address %d, file has %d bytes" % (self.eof, len(b)))
        root = self._entry(56)
        self.root_header = root["header"]
        msgs = self.object_header(self.root_header)
        st = [m for m in msgs if m.type == 0x11]
        if len(st) != 1:
            raise Hdf5Error("root group without a symbol table message")
        btree, heap = struct.unpack_from("<QQ", st[0].data, 0)
        if root["cache"] == 1 and (root["btree"], root["heap"]) != (btree, heap):
            raise Hdf5Error("root entry scratch pad disagrees with its symbol table")
        self.heap = self._local_heap(heap)
        self.entries = {}
        self.btree_nodes = {}  # level -> [(address, left sibling, right sibling)]
        self._walk_btree(btree, None)
        self._check_siblings()
        self.datasets = {}
        for name, addr in self.entries.items():
            self.datasets[name] = self._dataset(name, addr)

    # -- structures -------------------------------------------------------
    def _entry(self, off):
        b = self.buf
        return {
            "name": _u(b, off, 8),
            "header": _u(b, off + 8, 8),
            "cache": _u(b, off + 16, 4),
            "btree": _u(b, off + 24, 8),
            "heap": _u(b, off + 32, 8),
        }

    def _local_heap(self, addr):
        b = self.buf
        if b[addr:addr + 4] != b"HEAP" or b[addr + 4] != 0:
            raise Hdf5Error("bad local heap at %d" % addr)
        size = _u(b, addr + 8, 8)
        data = _u(b, addr + 24, 8)
        return b[data:data + size]

    def heap_string(self, off):
        end = self.heap.index(b"\0", off)
        return self.heap[off:end].decode()

    def _walk_btree(self, addr, bounds):
        b = self.buf
        if b[addr:addr + 4] != b"TREE" or b[addr + 4] != 0:
            raise Hdf5Error("bad group B-tree node at %d" % addr)
        level = b[addr + 5]
        used = _u(b, addr + 6, 2)
        self.btree_nodes.setdefault(level, []).append(
            (addr, _u(b, addr + 8, 8), _u(b, addr + 16, 8)))
        if used > 2 * self.internal_k:
            raise Hdf5Error("B-tree node with %d entries" % used)
        off = addr + 24
        keys = []
        children = []
        for i in range(used):
            keys.append(_u(b, off, 8))
            children.append(_u(b, off + 8, 8))
            off += 16
        keys.append(_u(b, off, 8))
        for i, c in enumerate(children):
            lo = self.heap_string(keys[i])
            hi = self.heap_string(keys[i + 1])
            if level > 0:
                self._walk_btree(c, (lo, hi))
            else:
                self._snod(c, lo, hi)

    def _check_siblings(self):
        """Nodes of one level, visited left to right, link to each other."""
        for level, nodes in self.btree_nodes.items():
            for q, (addr, left, right) in enumerate(nodes):
                want_left = nodes[q - 1][0] if q > 0 else UNDEF
                want_right = nodes[q + 1][0] if q + 1 < len(nodes) else UNDEF
                if (left, right) != (want_left, want_right):
                    raise Hdf5Error("B-tree node %d at level %d: bad sibling links" % (addr, level))

    def _snod(self, addr, lo, hi):
        b = self.buf
        if b[addr:addr + 4] != b"SNOD" or b[addr + 4] != 1:
            raise Hdf5Error("bad symbol table node at %d" % addr)
        n = _u(b, addr + 6, 2)
        if n > 2 * self.leaf_k:
            raise Hdf5Error("symbol table node with %d entries" % n)
        prev = None
        for s in range(n):
            e = self._entry(addr + 8 + 40 * s)
            name = self.heap_string(e["name"])
            # names in a node are sorted and lie in (key[i], key[i+1]]
            if prev is not None and not prev < name:
                raise Hdf5Error("names out of order: %r, %r" % (prev, name))
            if not (lo < name <= hi):
                raise Hdf5Error("name %r outside its node's keys (%r, %r]" % (name, lo, hi))
            if name in self.entries:
                raise Hdf5Error("duplicate name %r" % name)
            self.entries[name] = e["header"]
            prev = name

    def object_header(self, addr):
        b = self.buf
        if b[addr] != 1:
            raise Hdf5Error("object header version %d at %d" % (b[addr], addr))
        nmsg = _u(b, addr + 2, 2)
        size = _u(b, addr + 8, 4)
        chunks = [(addr + 16, size)]
        msgs = []
        while chunks:
            off, size = chunks.pop(0)
            end = off + size
            while off < end and len(msgs) < nmsg:
                mtype = _u(b, off, 2)
                msize = _u(b, off + 2, 2)
                flags = b[off + 4]
                if msize % 8:
                    raise Hdf5Error("message size %d not a multiple of 8" % msize)
                data = b[off + 8:off + 8 + msize]
                if mtype == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", data, 0)
                    chunks.append((caddr, clen))
                msgs.append(Message(mtype, flags, data))
                off += 8 + msize
            if off > end:
                raise Hdf5Error("messages overrun their chunk")
        if len(msgs) != nmsg:
            raise Hdf5Error("%d messages, header says %d" % (len(msgs), nmsg))
        return msgs

    def _dataset(self, name, addr):
        msgs = self.object_header(addr)
        by = {}
        for m in msgs:
            by.setdefault(m.type, m)
        for t in (0x01, 0x03, 0x08):
            if t not in by:
                raise Hdf5Error("dataset %r lacks message type %d" % (name, t))
        # dataspace
        d = by[0x01].data
        ver, rank, flags = d[0], d[1], d[2]
        if ver == 1:
            off = 8
        elif ver == 2:
            off = 4
        else:
            raise Hdf5Error("dataspace version %d" % ver)
        shape = tuple(_u(d, off + 8 * i, 8) for i in range(rank))
        # datatype
        t = by[0x03].data
        cls, tver = t[0] & 0x0F, t[0] >> 4
        bits = _u(t, 1, 3)
        size = _u(t, 4, 4)
        if bits & 1:
            raise Hdf5Error("big-endian datatype")
        if cls == 1:  # floating point
            if size == 4:
                dtype = np.dtype("<f4")
            elif size == 8:
                dtype = np.dtype("<f8")
            else:
                raise Hdf5Error("float of %d bytes" % size)
            boff, prec, eloc, esz, mloc, msz, bias = struct.unpack_from("<HHBBBBI", t, 8)
            ieee = {4: (0, 32, 23, 8, 0, 23, 127), 8: (0, 64, 52, 11, 0, 52, 1023)}[size]
            if (boff, prec, eloc, esz, mloc, msz, bias) != ieee:
                raise Hdf5Error("non-IEEE float layout")
        elif cls == 0:  # fixed point
            signed = bool(bits & 8)
            dtype = np.dtype(("<i%d" if signed else "<u%d") % size)
        else:
            raise Hdf5Error("datatype class %d" % cls)
        # layout
        l = by[0x08].data
        if l[0] != 3:
            raise Hdf5Error("layout version %d" % l[0])
        if l[1] == 1:
            daddr, nbytes = struct.unpack_from("<QQ", l, 2)
        else:
            raise Hdf5Error("layout class %d (only contiguous is read)" % l[1])
        count = int(np.prod(shape)) if shape else 1
        if nbytes != count * dtype.itemsize:
            raise Hdf5Error("dataset %r: %d bytes for %d elements" % (name, nbytes, count))
        if daddr != UNDEF and daddr + nbytes > len(self.buf):
            raise Hdf5Error("dataset %r runs past the end of the file" % name)
        return Dataset(name, shape, dtype, daddr, nbytes, msgs)

    # -- access -------------------------------------------------------------
    def keys(self):
        return sorted(self.datasets)

    def __contains__(self, name):
        return name in self.datasets

    def __getitem__(self, name):
        d = self.datasets[name]
        if d.addr == UNDEF:
            return np.zeros(d.shape, d.dtype)
        a = np.frombuffer(self.buf, d.dtype, d.nbytes // d.dtype.itemsize, d.addr)
        return a.reshape(d.shape).copy()

    def message_types(self, name):
        return [m.type for m in self.datasets[name].messages]
