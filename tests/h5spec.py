"""An independent, test-only restatement of the parts of the HDF5 file format
(specification: superblock versions 0/1, version-1 object headers,
symbol-table groups with version-1 B-trees and local heaps, dataspace,
datatype and layout messages) that the library's own reader and writer
(meshlesshydro_gb300/csrc/mlh_io.cpp) use.

`read` parses files the library writes; `write_variant` writes files with
the structures HDF5 itself produces for larger or older files that the
library's writer never emits (a two-level group B-tree over several symbol
table nodes, continuation blocks, NIL and unknown messages, compact storage,
big-endian and narrow types, version-2 dataspaces, superblock version 1), so
that the library's reader is checked against a second implementation.
"""
import struct

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


def _u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def read(path):
    """{name: numpy array} of the root group's datasets."""
    b = open(path, "rb").read()
    assert b[:8] == SIG
    ver = b[8]
    so, sl = b[13], b[14]
    p = 24 + (4 if ver == 1 else 0) + 4 * so
    root_oh = _u(b, p + so, so)

    def messages(addr):
        assert b[addr] == 1
        n = _u(b, addr + 2, 2)
        blocks = [(addr + 16, _u(b, addr + 8, 4))]
        out = []
        while blocks and len(out) < n:
            start, size = blocks.pop(0)
            q = start
            while q + 8 <= start + size and len(out) < n:
                t, sz = _u(b, q, 2), _u(b, q + 2, 2)
                data = b[q + 8:q + 8 + sz]
                out.append((t, data))
                if t == 0x10:
                    blocks.append((_u(data, 0, so), _u(data, so, sl)))
                q += 8 + sz
        return out

    btree = heap = None
    for t, d in messages(root_oh):
        if t == 0x11:
            btree, heap = _u(d, 0, so), _u(d, so, so)
    assert b[heap:heap + 4] == b"HEAP"
    hdata = _u(b, heap + 8 + 2 * sl, so)
    names = {}

    def walk(node):
        assert b[node:node + 4] == b"TREE" and b[node + 4] == 0
        level, used = b[node + 5], _u(b, node + 6, 2)
        for k in range(used):
            child = _u(b, node + 8 + 2 * so + k * (sl + so) + sl, so)
            if level > 0:
                walk(child)
                continue
            assert b[child:child + 4] == b"SNOD"
            for e in range(_u(b, child + 6, 2)):
                ent = child + 8 + e * (2 * so + 24)
                off = _u(b, ent, so)
                end = b.index(b"\0", hdata + off)
                names[b[hdata + off:end].decode()] = _u(b, ent + so, so)

    walk(btree)
    out = {}
    for name, oh in names.items():
        shape, dtype, data = None, None, None
        for t, d in messages(oh):
            if t == 1:
                rank = d[1]
                q = 8 if d[0] == 1 else 4
                shape = tuple(_u(d, q + 8 * k, 8) for k in range(rank))
            elif t == 3:
                cls, size = d[0] & 15, _u(d, 4, 4)
                order = ">" if d[1] & 1 else "<"
                kind = "f" if cls == 1 else ("i" if d[1] & 8 else "u")
                dtype = np.dtype(f"{order}{kind}{size}")
            elif t == 8:
                assert d[0] == 3
                if d[1] == 1:
                    addr, size = _u(d, 2, so), _u(d, 2 + so, sl)
                    data = b[addr:addr + size]
                else:
                    data = d[4:4 + _u(d, 2, 2)]
        out[name] = np.frombuffer(data, dtype=dtype).reshape(shape)
    return out


class _Buf:
    def __init__(self):
        self.b = bytearray()

    def at(self):
        return len(self.b)

    def put(self, data):
        self.b += data

    def pad(self, n=8):
        while len(self.b) % n:
            self.b.append(0)

    def reserve(self, n):
        a = len(self.b)
        self.b += bytes(n)
        return a

    def patch(self, off, data):
        self.b[off:off + len(data)] = data


def _dtype_msg(dt):
    dt = np.dtype(dt)
    be = 1 if dt.byteorder == ">" else 0
    if dt.kind == "f":
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            bits = bytes([0x20 | be, 63, 0])
        else:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            bits = bytes([0x20 | be, 31, 0])
        return bytes([0x11]) + bits + struct.pack("<I", dt.itemsize) + props
    signed = 8 if dt.kind == "i" else 0
    return bytes([0x10, signed | be, 0, 0]) + struct.pack("<IHH", dt.itemsize, 0, 8 * dt.itemsize)


def _msg(t, data, flags=0):
    data = bytes(data)
    data += bytes((-len(data)) % 8)
    return struct.pack("<HHB3x", t, len(data), flags) + data


def write_variant(path, datasets, leaf_k=2):
    """Writes {name: array} with superblock version 1, a two-level group
    B-tree over several symbol table nodes (leaf_k sets their capacity to
    2 * leaf_k), object headers split by a continuation message with NIL and
    unknown messages, arrays of 16 bytes or less in compact storage, others
    contiguous; every dtype is kept as given."""
    names = sorted(datasets)
    buf = _Buf()
    sb = buf.reserve(24 + 4 + 4 * 8 + 40)
    root = buf.at()
    buf.put(struct.pack("<BBHII4x", 1, 0, 1, 1, 24))
    root_msg = buf.reserve(24)
    buf.pad()
    heap_data = bytearray(bytes(8))
    offs = {}
    for n in names:
        offs[n] = len(heap_data)
        heap_data += n.encode() + b"\0"
        heap_data += bytes((-len(heap_data)) % 8)
    heap = buf.at()
    buf.put(b"HEAP" + bytes(4) + struct.pack("<QQQ", len(heap_data), 1, heap + 32))
    buf.put(heap_data)
    buf.pad()
    # dataset object headers and data
    oh = {}
    for n in names:
        a = np.ascontiguousarray(datasets[n])
        space_v2 = a.ndim == 1
        if space_v2:
            space = bytes([2, a.ndim, 0, 1]) + b"".join(struct.pack("<Q", d) for d in a.shape)
        else:
            space = bytes([1, a.ndim, 0, 0, 0, 0, 0, 0]) + b"".join(struct.pack("<Q", d) for d in a.shape)
        raw = a.tobytes()
        compact = len(raw) <= 16
        first = [_msg(0x0000, bytes(16)), _msg(0x0001, space), _msg(0x0003, _dtype_msg(a.dtype), 1),
                 _msg(0x0012, struct.pack("<BxxxI", 1, 1700000000))]
        cont_at = None
        second_msgs = []
        if compact:
            second_msgs.append(_msg(0x0008, bytes([3, 0]) + struct.pack("<H", len(raw)) + raw))
        else:
            second_msgs.append(None)   # layout, address patched below
        second_msgs.append(_msg(0x00C0, b"unknown message body"))
        layout_len = len(_msg(0x0008, bytes(18)))
        second_size = sum(len(m) if m is not None else layout_len for m in second_msgs)
        header = b"".join(first)
        hdr_at = buf.at()
        nmsgs = len(first) + 1 + len(second_msgs)
        buf.put(struct.pack("<BBHII4x", 1, 0, nmsgs, 1, len(header) + 24))
        buf.put(header)
        cont_at = buf.reserve(24)
        buf.pad()
        block = buf.at()
        layout_pos = None
        for m in second_msgs:
            if m is None:
                layout_pos = buf.reserve(layout_len)
            else:
                buf.put(m)
        buf.patch(cont_at, _msg(0x0010, struct.pack("<QQ", block, second_size)))
        buf.pad()
        if not compact:
            data_at = buf.at()
            buf.put(raw)
            buf.pad()
            buf.patch(layout_pos, _msg(0x0008, bytes([3, 1]) + struct.pack("<QQ", data_at, len(raw))))
        oh[n] = hdr_at
    # symbol table nodes of at most 2 * leaf_k links
    cap = 2 * leaf_k
    groups = [names[i:i + cap] for i in range(0, len(names), cap)]
    snods = []
    for g in groups:
        at = buf.at()
        buf.put(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(g)))
        for n in g:
            buf.put(struct.pack("<QQII16x", offs[n], oh[n], 0, 0))
        buf.put(bytes((cap - len(g)) * 40))
        snods.append((at, g[-1]))
    # two leaves under one internal node
    half = (len(snods) + 1) // 2
    leaves = []
    for part in (snods[:half], snods[half:]):
        if not part:
            continue
        at = buf.at()
        buf.put(b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(part), UNDEF, UNDEF))
        buf.put(struct.pack("<Q", 0))
        for child, last in part:
            buf.put(struct.pack("<QQ", child, offs[last]))
        leaves.append((at, part[-1][1]))
    top = buf.at()
    buf.put(b"TREE" + bytes([0, 1]) + struct.pack("<HQQ", len(leaves), UNDEF, UNDEF))
    buf.put(struct.pack("<Q", 0))
    for child, last in leaves:
        buf.put(struct.pack("<QQ", child, offs[last]))
    buf.patch(root_msg, _msg(0x0011, struct.pack("<QQ", top, heap)))
    eof = buf.at()
    sbb = SIG + bytes([1, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHIHH", leaf_k, 16, 0, 32, 0)
    sbb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
    sbb += struct.pack("<QQII", 0, root, 1, 0) + struct.pack("<QQ", top, heap)
    buf.patch(sb, sbb)
    with open(path, "wb") as f:
        f.write(buf.b)
