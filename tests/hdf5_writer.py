"""A small HDF5 writer for the reader's tests (classic file format, as the library
writes with its default properties): superblock version 0, version 1 object headers,
symbol-table groups, contiguous / compact / chunked datasets (deflate, shuffle and
Fletcher-32 filters, one- or two-level chunk B-trees), version 1 attribute messages,
optional continuation blocks and user block.  Test infrastructure only: the reader is
pinned to real files by tests/golden/hdf5/; this covers the structures those files lack.

    w = H5Writer()
    w.dataset("PartType0/Masses", masses, attrs={"to_cgs": 1.989e43, ...})
    w.write(path)
"""
from __future__ import annotations

import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


def _datatype(dtype: np.dtype, version: int = 0) -> bytes:
    """Datatype message of a numpy dtype; `version` picks the encoding of compound (1, 2
    or 3; default 1) and array (2 or 3; default 2) types."""
    dtype = np.dtype(dtype)
    if dtype.subdtype is not None:  # array class
        base, dims = dtype.subdtype
        v = version or 2
        head = bytes([0x0A | (v << 4), 0, 0, 0]) + struct.pack("<I", dtype.itemsize) + bytes([len(dims)])
        if v == 2:
            head += b"\0" * 3 + b"".join(struct.pack("<I", d) for d in dims) + \
                b"".join(struct.pack("<I", i) for i in range(len(dims)))
        else:
            head += b"".join(struct.pack("<I", d) for d in dims)
        return head + _datatype(base, version)
    if dtype.names:  # compound class
        v = version or 1
        size = dtype.itemsize
        body = b""
        for name in dtype.names:
            member, offset = dtype.fields[name][:2]
            nm = name.encode() + b"\0"
            if v < 3:
                body += _pad8(nm) + struct.pack("<I", offset)
                if v == 1:
                    body += bytes([0, 0, 0, 0]) + b"\0" * 4 + b"\0" * 4 + b"\0" * 16
            else:
                nbytes = 1 if size < 1 << 8 else 2 if size < 1 << 16 else 3 if size < 1 << 24 else 4
                body += nm + offset.to_bytes(nbytes, "little")
            body += _datatype(member, version if member.names or member.subdtype else 0)
        n = len(dtype.names)
        return bytes([0x06 | (v << 4), n & 0xFF, n >> 8, 0]) + struct.pack("<I", size) + body
    be = 1 if dtype.byteorder == ">" or (dtype.byteorder == "=" and np.little_endian is False) else 0
    size = dtype.itemsize
    if dtype.kind in "iu":
        bits = be | (8 if dtype.kind == "i" else 0)
        return bytes([0x10, bits, 0, 0]) + struct.pack("<IHH", size, 0, 8 * size)
    if dtype.kind == "f":
        layout = {2: (10, 5, 10, 15), 4: (23, 8, 23, 127), 8: (52, 11, 52, 1023)}[size]
        sign = 8 * size - 1
        return bytes([0x11, be | 0x20, sign, 0]) + struct.pack("<IHHBBBBI", size, 0, 8 * size, layout[0],
                                                                layout[1], 0, layout[2], layout[3])
    if dtype.kind == "S":
        return bytes([0x13, 0, 0, 0]) + struct.pack("<I", size)
    raise TypeError(dtype)


def _dataspace(shape, version=1) -> bytes:
    if version == 1:
        out = bytes([1, len(shape), 1 if shape else 0, 0]) + b"\0" * 4
        for d in shape:
            out += struct.pack("<Q", d)
        for d in shape:
            out += struct.pack("<Q", d)
        return out
    out = bytes([2, len(shape), 1 if shape else 0, 1 if shape else 0])
    for d in shape:
        out += struct.pack("<Q", d)
    for d in shape:
        out += struct.pack("<Q", d)
    return out


def _message(mtype: int, data: bytes, flags: int = 0) -> bytes:
    data = _pad8(data)
    return struct.pack("<HHB3x", mtype, len(data), flags) + data


class VlenString:
    """An attribute holding one variable-length string (datatype class 9): written with
    a null global-heap reference, enough for a reader that does not decode it."""

    def __init__(self, text: str):
        self.text = text


def _attribute(name: str, value) -> bytes:
    nm = name.encode() + b"\0"
    if isinstance(value, VlenString):
        # class 9 version 1, type 1 (string), null-terminated ASCII; base type: 1-byte char
        dt = bytes([0x19, 0x01, 0, 0]) + struct.pack("<I", 16) + bytes([0x13, 0, 0, 0]) + struct.pack("<I", 1)
        ds = _dataspace(())
        data = struct.pack("<IQI", len(value.text), 0, 0)
    else:
        value = np.asarray(value)
        dt = _datatype(value.dtype)
        ds = _dataspace(value.shape)
        data = value.tobytes()
    body = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds)) + _pad8(nm) + _pad8(dt) + _pad8(ds)
    return _message(0x0C, body + data)


def _shuffle(raw: bytes, width: int) -> bytes:
    k = len(raw) // width
    body = np.frombuffer(raw[:k * width], np.uint8).reshape(k, width).T.reshape(-1)
    return body.tobytes() + raw[k * width:]


class H5Writer:
    def __init__(self, user_block: int = 0, continuation: bool = False):
        self.tree = {"attrs": {}, "members": {}}
        self.user_block = user_block
        self.continuation = continuation
        self.buf = bytearray()

    # -- building the tree
    def _group(self, path: str) -> dict:
        node = self.tree
        for part in [p for p in path.strip("/").split("/") if p]:
            node = node["members"].setdefault(part, {"attrs": {}, "members": {}})
        return node

    def group(self, path: str, attrs=None):
        self._group(path)["attrs"].update(attrs or {})

    def dataset(self, path: str, data, attrs=None, layout="contiguous", chunks=None,
                filters=(), filter_mask_first_chunk=0, btree_fanout=None, dataspace_version=1,
                layout_version=3, unallocated=False, dtype=None, type_version=0):
        """`dtype`: the element type when it is an array type (numpy folds a subarray
        dtype into the data's shape, so it is given apart)."""
        parent, _, name = path.strip("/").rpartition("/")
        self._group(parent)["members"][name] = {
            "data": np.asarray(data), "attrs": dict(attrs or {}), "layout": layout, "chunks": chunks,
            "filters": tuple(filters), "mask0": filter_mask_first_chunk, "fanout": btree_fanout,
            "dsv": dataspace_version, "lv": layout_version, "unallocated": unallocated,
            "dtype": None if dtype is None else np.dtype(dtype), "tv": type_version}

    # -- serialising
    def _append(self, b: bytes) -> int:
        """Append at an 8-byte boundary; returns the address relative to the base."""
        self.buf += b"\0" * (-len(self.buf) % 8)
        at = len(self.buf)
        self.buf += b
        return at - self.user_block

    def _header(self, messages) -> int:
        if self.continuation and len(messages) > 2:
            head, tail = messages[:1], messages[1:]
            tail_bytes = b"".join(tail)
            cont_at = self._append(tail_bytes)
            head = head + [_message(0x10, struct.pack("<QQ", cont_at, len(tail_bytes)))]
            body = b"".join(head)
            count = len(messages) + 1
        else:
            body = b"".join(messages)
            count = len(messages)
        return self._append(struct.pack("<BBHII4x", 1, 0, count, 1, len(body)) + body)

    def _filters_message(self, filters, elem):
        body = struct.pack("<BB6x", 1, len(filters))
        for f in filters:
            if isinstance(f, int):  # a bare filter id without client data (nothing encoded)
                vals, fid = [], f
            else:
                vals = {"deflate": [6], "shuffle": [elem], "fletcher32": []}[f]
                fid = {"deflate": 1, "shuffle": 2, "fletcher32": 3}[f]
            body += struct.pack("<HHHH", fid, 0, 0, len(vals))
            body += b"".join(struct.pack("<I", v) for v in vals)
            if len(vals) % 2:
                body += b"\0" * 4
        return _message(0x0B, body)

    def _encode_chunk(self, raw: bytes, filters, elem, skip: int) -> bytes:
        for i, f in enumerate(filters):
            if skip & (1 << i):
                continue
            if f == "shuffle":
                raw = _shuffle(raw, elem)
            elif f == "deflate":
                raw = zlib.compress(raw, 6)
            elif f == "fletcher32":
                raw = raw + struct.pack("<I", zlib.adler32(raw))  # the reader only strips it
        return raw

    def _chunk_tree(self, entries, rank, fanout):
        """Type 1 B-tree over (offsets, size, mask, address) entries; returns its address."""
        def node(level, items):
            body = b"TREE" + struct.pack("<BBHQQ", 1, level, len(items), UNDEF, UNDEF)
            for offsets, size, mask, child in items:
                body += struct.pack("<II", size, mask) + b"".join(struct.pack("<Q", o) for o in offsets)
                body += struct.pack("<Q", child)
            body += struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", 0) for _ in range(rank + 1))
            return self._append(body)

        if not fanout or len(entries) <= fanout:
            return node(0, entries)
        leaves = []
        for i in range(0, len(entries), fanout):
            part = entries[i:i + fanout]
            leaves.append((part[0][0], 0, 0, node(0, part)))
        return node(1, leaves)

    def _write_dataset(self, d) -> int:
        data = d["data"]
        etype = d["dtype"] if d["dtype"] is not None else data.dtype
        shape = data.shape[:data.ndim - len(etype.shape)]
        raw = np.ascontiguousarray(data).tobytes()
        elem = etype.itemsize
        msgs = [_message(0x01, _dataspace(shape, d["dsv"])), _message(0x03, _datatype(etype, d["tv"]))]
        if d["layout"] == "contiguous":
            addr = UNDEF if (d["unallocated"] or not raw) else self._append(raw)
            if d["lv"] == 3:
                msgs.append(_message(0x08, struct.pack("<BBQQ", 3, 1, addr, len(raw))))
            else:
                body = struct.pack("<BBB5xQ", d["lv"], len(shape) + 1, 1, addr)
                body += b"".join(struct.pack("<I", s) for s in shape) + struct.pack("<I", elem)
                msgs.append(_message(0x08, body))
        elif d["layout"] == "compact":
            msgs.append(_message(0x08, struct.pack("<BBH", 3, 0, len(raw)) + raw))
        else:
            chunks = tuple(d["chunks"])
            entries = []
            grid = [range(0, s, c) for s, c in zip(shape, chunks)]
            for k, origin in enumerate(np.ndindex(*[len(g) for g in grid])):
                offsets = [g[i] for g, i in zip(grid, origin)]
                block = np.zeros(tuple(chunks) + etype.shape, data.dtype)
                src = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offsets, chunks, shape))
                block[tuple(slice(0, x.stop - x.start) for x in src)] = data[src]
                mask = d["mask0"] if k == 0 else 0
                enc = self._encode_chunk(block.tobytes(), d["filters"], elem, mask)
                entries.append((offsets + [0], len(enc), mask, self._append(enc)))
            tree = self._chunk_tree(entries, len(shape), d["fanout"]) if entries else UNDEF
            body = struct.pack("<BBBQ", 3, 2, len(shape) + 1, tree)
            body += b"".join(struct.pack("<I", c) for c in chunks) + struct.pack("<I", elem)
            msgs.append(_message(0x08, body))
            if d["filters"]:
                msgs.append(self._filters_message(d["filters"], elem))
        msgs += [_attribute(k, v) for k, v in d["attrs"].items()]
        return self._header(msgs)

    def _write_group(self, g) -> int:
        names = sorted(g["members"])
        children = {}
        for name in names:
            m = g["members"][name]
            children[name] = self._write_dataset(m) if "data" in m else self._write_group(m)
        heap = b"\0" * 8
        offsets = {}
        for name in names:
            offsets[name] = len(heap)
            heap += _pad8(name.encode() + b"\0")
        heap_data = self._append(heap)
        heap_at = self._append(b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap), UNDEF, heap_data))
        # symbol nodes of at most 2 * leaf K = 8 entries, as the library splits them; a
        # tree node holds at most 2 * internal K = 32 children, so larger groups get a
        # second level
        leaves = []  # (address, heap offset of the node's last name)
        for i in range(0, max(len(names), 1), 8):
            part = names[i:i + 8]
            snod = b"SNOD" + struct.pack("<BBH", 1, 0, len(part))
            for name in part:
                snod += struct.pack("<QQII16x", offsets[name], children[name], 0, 0)
            leaves.append((self._append(snod), offsets[part[-1]] if part else 0))

        def node(level, kids):
            body = b"TREE" + struct.pack("<BBHQQ", 0, level, len(kids), UNDEF, UNDEF) + struct.pack("<Q", 0)
            for addr, last in kids:
                body += struct.pack("<QQ", addr, last)
            return self._append(body)

        if len(leaves) <= 32:
            tree = node(0, leaves)
        else:
            tree = node(1, [(node(0, leaves[i:i + 32]), leaves[min(i + 32, len(leaves)) - 1][1])
                            for i in range(0, len(leaves), 32)])
        msgs = [_message(0x11, struct.pack("<QQ", tree, heap_at))]
        msgs += [_attribute(k, v) for k, v in g["attrs"].items()]
        return self._header(msgs)

    def write(self, path):
        self.buf = bytearray(b"\0" * self.user_block)
        sb_at = self._append(b"\0" * 96)  # superblock placeholder
        root = self._write_group(self.tree)
        eof = len(self.buf) - self.user_block
        sb = b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
        sb += struct.pack("<QQQQ", self.user_block, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQII16x", 0, root, 0, 0)
        start = sb_at + self.user_block
        self.buf[start:start + 96] = sb
        with open(path, "wb") as f:
            f.write(self.buf)
