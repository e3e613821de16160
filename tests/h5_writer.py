"""A minimal HDF5 writer for the tests of the library's HDF5 mesh reader.

It writes the layout CHM's own mesh and parameter files use: superblock
version 0, groups in symbol tables (a one-node version-1 B-tree, one
symbol-table node, a local heap), version-1 object headers, contiguous
one-dimensional datasets of fixed-point, floating-point or 3-element array
types, and attributes on the root group whose names contain slashes
("/mesh/version", ...), with fixed-length strings.  Written from the
published HDF5 file-format specification; test infrastructure only.
"""
from __future__ import annotations

import struct

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


class _Buf:
    def __init__(self):
        self.b = bytearray()

    def alloc(self, n: int, align: int = 8) -> int:
        while len(self.b) % align:
            self.b.append(0)
        a = len(self.b)
        self.b.extend(b"\0" * n)
        return a

    def put(self, addr: int, data: bytes):
        self.b[addr:addr + len(data)] = data


def _pad8(x: bytes) -> bytes:
    return x + b"\0" * (-len(x) % 8)


def _fixed_type(size: int, signed: bool, big: bool = False) -> bytes:
    bits = (1 if big else 0) | (8 if signed else 0)
    return bytes([0x10, bits, 0, 0]) + struct.pack("<I", size) + struct.pack("<HH", 0, 8 * size)


def _float_type(size: int = 8, big: bool = False) -> bytes:
    if size == 8:
        props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
        bits = 0x20 | (1 if big else 0)
        return bytes([0x11, bits, 0x3F, 0]) + struct.pack("<I", 8) + props
    props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
    return bytes([0x11, 0x20 | (1 if big else 0), 0x1F, 0]) + struct.pack("<I", 4) + props


def _array_type(base: bytes, n: int, base_size: int) -> bytes:
    # version 2 array: rank, 3 reserved bytes, dims, permutation indices, base type
    return bytes([0x2A, 0, 0, 0]) + struct.pack("<I", n * base_size) + bytes([1, 0, 0, 0]) + \
        struct.pack("<I", n) + struct.pack("<I", 0) + base


def _string_type(size: int) -> bytes:
    return bytes([0x13, 0, 0, 0]) + struct.pack("<I", size)


def _space(n: int) -> bytes:
    return bytes([1, 1, 1, 0, 0, 0, 0, 0]) + struct.pack("<QQ", n, n)


def _scalar_space() -> bytes:
    return bytes([1, 1, 1, 0, 0, 0, 0, 0]) + struct.pack("<QQ", 1, 1)


def _msg(mtype: int, body: bytes) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), 0) + body


def _ohdr(buf: _Buf, msgs: list[bytes]) -> int:
    body = b"".join(msgs)
    addr = buf.alloc(16 + len(body))
    buf.put(addr, struct.pack("<BBHII", 1, 0, len(msgs), 1, len(body)) + b"\0" * 4 + body)
    return addr


def _attribute(name: str, dtype: bytes, space: bytes, data: bytes) -> bytes:
    nm = name.encode() + b"\0"
    return struct.pack("<BBHHH", 1, 0, len(nm), len(dtype), len(space)) + _pad8(nm) + _pad8(dtype) + \
        _pad8(space) + data


def _group(buf: _Buf, members: dict[str, tuple[int, tuple[int, int] | None]], extra_msgs=()) -> tuple:
    """Local heap + B-tree + symbol-table node for members {name: (object
    header address, (btree, heap) when the member is a group)}; returns the
    group's (object header, btree, heap)."""
    names = sorted(members)
    heap_data = bytearray(b"\0" * 8)  # offset 0: the empty name
    offs = {}
    for n in names:
        offs[n] = len(heap_data)
        heap_data += _pad8(n.encode() + b"\0")
    data_addr = buf.alloc(len(heap_data))
    buf.put(data_addr, bytes(heap_data))
    heap = buf.alloc(32)
    buf.put(heap, b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), UNDEF, data_addr))
    ents = b""
    for n in names:
        oh, sub = members[n]
        if sub is None:
            ents += struct.pack("<QQII", offs[n], oh, 0, 0) + b"\0" * 16
        else:
            ents += struct.pack("<QQII", offs[n], oh, 1, 0) + struct.pack("<QQ", sub[0], sub[1])
    snod = buf.alloc(8 + len(ents))
    buf.put(snod, b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names)) + ents)
    tree = buf.alloc(8 + 16 + 8 + 8 + 8)
    last = offs[names[-1]] if names else 0
    buf.put(tree, b"TREE" + bytes([0, 0]) + struct.pack("<H", 1) + struct.pack("<QQ", UNDEF, UNDEF) +
            struct.pack("<QQQ", 0, snod, last))
    oh = _ohdr(buf, [_msg(0x11, struct.pack("<QQ", tree, heap))] + list(extra_msgs))
    return oh, tree, heap


def _dataset(buf: _Buf, arr: np.ndarray, kind: str) -> int:
    """kind: "f64", "i32", "i32be", "f64x3", "i32x3"."""
    n = arr.shape[0]
    if kind == "f64":
        dtype, raw = _float_type(8), arr.astype("<f8").tobytes()
    elif kind == "i32":
        dtype, raw = _fixed_type(4, True), arr.astype("<i4").tobytes()
    elif kind == "i32be":
        dtype, raw = _fixed_type(4, True, big=True), arr.astype(">i4").tobytes()
    elif kind == "f64x3":
        dtype, raw = _array_type(_float_type(8), 3, 8), arr.astype("<f8").tobytes()
    elif kind == "i32x3":
        dtype, raw = _array_type(_fixed_type(4, True), 3, 4), arr.astype("<i4").tobytes()
    else:
        raise ValueError(kind)
    data = buf.alloc(len(raw))
    buf.put(data, raw)
    layout = bytes([3, 1]) + struct.pack("<QQ", data, len(raw))
    return _ohdr(buf, [_msg(0x1, _space(n)), _msg(0x3, dtype), _msg(0x8, layout)])


def _file(build) -> bytes:
    buf = _Buf()
    buf.alloc(24 + 32 + 40)  # superblock, written last
    root_oh, tree, heap, eof = build(buf)
    sb = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
    sb += struct.pack("<QQQQ", 0, UNDEF, len(buf.b), UNDEF)
    sb += struct.pack("<QQII", 0, root_oh, 1, 0) + struct.pack("<QQ", tree, heap)
    buf.put(0, sb)
    return bytes(buf.b)


def write_mesh_h5(path, xyz, tri, neighbor, version="2.0.0", is_geographic=0, is_partition=0,
                  global_ids=None, proj4="+proj=utm +zone=8 +datum=NAD83 +units=m +no_defs"):
    nt = len(tri)
    gid = np.arange(nt) if global_ids is None else np.asarray(global_ids)

    def build(buf):
        members = {"vertex": (_dataset(buf, np.asarray(xyz, float), "f64x3"), None),
                   "elem": (_dataset(buf, np.asarray(tri), "i32x3"), None),
                   "neighbor": (_dataset(buf, np.asarray(neighbor), "i32x3"), None),
                   "cell_global_id": (_dataset(buf, gid, "i32be"), None),
                   "local_sizes": (_dataset(buf, np.array([nt]), "i32be"), None)}
        moh, mtree, mheap = _group(buf, members)

        def s(v):
            return _string_type(256), (v.encode() + b"\0").ljust(256, b"\0")
        attrs = []
        for name, (dt, data) in {"/mesh/proj4": s(proj4), "/mesh/version": s(version),
                                 "/mesh/partition_method": s("metis")}.items():
            attrs.append(_msg(0xC, _attribute(name, dt, _scalar_space(), data)))
        for name, v in (("/mesh/is_geographic", is_geographic), ("/mesh/is_partition", is_partition)):
            attrs.append(_msg(0xC, _attribute(name, _fixed_type(1, False), _scalar_space(), bytes([v]))))
        roh, rtree, rheap = _group(buf, {"mesh": (moh, (mtree, mheap))}, attrs)
        return roh, rtree, rheap, len(buf.b)
    open(path, "wb").write(_file(build))


def write_params_h5(path, params: dict):
    def build(buf):
        members = {k: (_dataset(buf, np.asarray(v, float), "f64"), None) for k, v in params.items()}
        poh, ptree, pheap = _group(buf, members)
        roh, rtree, rheap = _group(buf, {"parameters": (poh, (ptree, pheap))})
        return roh, rtree, rheap, len(buf.b)
    open(path, "wb").write(_file(build))
