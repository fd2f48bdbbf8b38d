"""Read-only HDF5 for the sweep's input files, in numpy (no libhdf5 or h5py needed).

Covers the classic file format that Arepo and the reference's own writer (hdf5-rust
with the library's default, earliest-format properties) produce:

* superblock versions 0 and 1 (with or without a user block in front);
* version 1 object headers, with continuation blocks;
* groups stored as symbol tables (version 1 B-tree of type 0, symbol nodes, local heap);
* dataspaces (versions 1 and 2: scalar, simple, null);
* fixed-point and IEEE floating-point datatypes of either byte order, fixed-length
  strings, and compound and array types built from them;
* data layouts of versions 1 to 3: compact, contiguous, and chunked (version 1 B-tree of
  type 1) with the deflate, shuffle and Fletcher-32 filters;
* attribute messages of versions 1 to 3 (stored in the object header).

Files that need the format's newer structures (superblock 2/3, version 2 object
headers, link messages, fractal heaps, version 4 layouts, dense attribute storage,
shared or committed datatypes) are rejected with `H5Error` naming the structure;
an attribute of a type the reader does not decode reads as None.

On top of the reader, `read_dataset` restates the reference's dataset input
(src/io/input/mod.rs:260-299 `read_region_chunked`, `get_dataset_and_conversion_factor_for_file`,
`convert_dataset_units`) with its three unit readers: the reference's own attributes
(src/io/unit_reader.rs:37-67 `DefaultUnitReader`), none (`IdReader`, :69-80) and
Arepo's (src/arepo_postprocess/unit_reader.rs:45-128 `ArepoUnitReader`).
"""
from __future__ import annotations

import dataclasses
import mmap
import os
import pathlib
import zlib
from typing import Optional, Sequence, Tuple, Union

import numpy as np

from .cosmology import Cosmology  # noqa: F401  (the unit readers' cosmology)

SIGNATURE = b"\x89HDF\r\n\x1a\n"


class H5Error(ValueError):
    """A file this reader cannot read, or a dataset or attribute that is missing."""


# header message types (HDF5 file format specification, section IV.A.2)
_MSG_NIL, _MSG_DATASPACE, _MSG_LINK_INFO, _MSG_DATATYPE = 0x0, 0x1, 0x2, 0x3
_MSG_LAYOUT, _MSG_LINK, _MSG_FILTERS, _MSG_ATTRIBUTE = 0x8, 0x6, 0xB, 0xC
_MSG_CONTINUATION, _MSG_SYMBOL_TABLE, _MSG_ATTRIBUTE_INFO = 0x10, 0x11, 0x15

_FILTER_DEFLATE, _FILTER_SHUFFLE, _FILTER_FLETCHER32 = 1, 2, 3


class _Reader:
    """Little-endian field access into the mapped file, with the superblock's sizes."""

    def __init__(self, buf, base: int, size_offsets: int, size_lengths: int):
        self.buf = buf
        self.base = base
        self.so = size_offsets
        self.sl = size_lengths
        self.undefined = (1 << (8 * size_offsets)) - 1

    def u(self, pos: int, n: int) -> int:
        if pos < 0 or pos + n > len(self.buf):
            raise H5Error(f"read of {n} bytes at {pos} past the end of the file ({len(self.buf)} bytes)")
        return int.from_bytes(self.buf[pos:pos + n], "little")

    def raw(self, pos: int, n: int) -> bytes:
        if pos < 0 or pos + n > len(self.buf):
            raise H5Error(f"read of {n} bytes at {pos} past the end of the file ({len(self.buf)} bytes)")
        return bytes(self.buf[pos:pos + n])

    def array(self, pos: int, dtype: np.dtype, count: int) -> np.ndarray:
        """A view of `count` elements at pos (valid while the file is open)."""
        if pos < 0 or pos + count * dtype.itemsize > len(self.buf):
            raise H5Error(f"data of {count * dtype.itemsize} bytes at {pos} past the end of the file")
        return np.frombuffer(self.buf, dtype=dtype, count=count, offset=pos)

    def addr(self, pos: int) -> Optional[int]:
        """File address stored at pos (None when undefined), made absolute."""
        a = self.u(pos, self.so)
        return None if a == self.undefined else a + self.base

    def length(self, pos: int) -> int:
        return self.u(pos, self.sl)

    def cstring(self, pos: int) -> str:
        end = self.buf.find(b"\0", pos)
        if end < 0:
            raise H5Error(f"unterminated name at {pos}")
        return bytes(self.buf[pos:end]).decode("utf-8")


@dataclasses.dataclass
class _Message:
    type: int
    flags: int
    pos: int   # absolute position of the message data
    size: int


# ---------------------------------------------------------------------------------------
# datatypes and dataspaces

def _datatype(r: _Reader, pos: int) -> np.dtype:
    """numpy dtype of a datatype message (specification IV.A.2.d)."""
    return _datatype_at(r, pos)[0]


def _datatype_at(r: _Reader, pos: int) -> Tuple[np.dtype, int]:
    """(numpy dtype, encoded length in bytes) of the datatype description at pos."""
    cv = r.u(pos, 1)
    cls, version, bits, size = cv & 0x0F, cv >> 4, r.u(pos + 1, 3), r.u(pos + 4, 4)
    if cls == 0:  # fixed-point: bit 0 byte order, bit 3 signed; offset, precision
        order = ">" if bits & 1 else "<"
        offset, precision = r.u(pos + 8, 2), r.u(pos + 10, 2)
        if size not in (1, 2, 4, 8) or offset != 0 or precision != 8 * size:
            raise H5Error(f"fixed-point type of {size} bytes with bit offset {offset}, precision {precision}")
        return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}"), 12
    if cls == 1:  # floating-point: bit 0 byte order (bit 6: VAX order)
        if bits & 0x40:
            raise H5Error("VAX-order floating-point type")
        layouts = {2: (0, 16, 10, 5, 0, 10, 15), 4: (0, 32, 23, 8, 0, 23, 127),
                   8: (0, 64, 52, 11, 0, 52, 1023)}
        got = (r.u(pos + 8, 2), r.u(pos + 10, 2), r.u(pos + 12, 1), r.u(pos + 13, 1), r.u(pos + 14, 1),
               r.u(pos + 15, 1), r.u(pos + 16, 4))
        if layouts.get(size) != got:
            raise H5Error(f"floating-point type of {size} bytes that is not IEEE 754 binary{8 * size}")
        return np.dtype(f"{'>' if bits & 1 else '<'}f{size}"), 20
    if cls == 3:  # fixed-length string
        return np.dtype(f"S{size}"), 8
    if cls == 6:  # compound: members by name, byte offset and type
        names, formats, offsets = [], [], []
        p = pos + 8
        offset_bytes = 1 if size < 1 << 8 else 2 if size < 1 << 16 else 3 if size < 1 << 24 else 4
        for _ in range(bits & 0xFFFF):
            end = r.buf.find(b"\0", p)
            if end < 0:
                raise H5Error(f"unterminated compound member name at {p}")
            names.append(bytes(r.buf[p:end]).decode("utf-8"))
            p = (p + ((end - p + 1 + 7) & ~7)) if version < 3 else end + 1
            if version < 3:
                offsets.append(r.u(p, 4))
                p += 4
            else:
                offsets.append(r.u(p, offset_bytes))
                p += offset_bytes
            dims = ()
            if version == 1:
                rank = r.u(p, 1)
                dims = tuple(r.u(p + 12 + 4 * i, 4) for i in range(rank))
                p += 28
            member, n = _datatype_at(r, p)
            p += n
            formats.append((member, dims) if dims else member)
        if not names:
            raise H5Error("compound datatype without members")
        return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size}), p - pos
    if cls == 10:  # array of a base type
        rank = r.u(pos + 8, 1)
        if version == 2:
            dims = tuple(r.u(pos + 12 + 4 * i, 4) for i in range(rank))
            p = pos + 12 + 8 * rank
        elif version == 3:
            dims = tuple(r.u(pos + 9 + 4 * i, 4) for i in range(rank))
            p = pos + 9 + 4 * rank
        else:
            raise H5Error(f"array datatype version {version}")
        base, n = _datatype_at(r, p)
        return np.dtype((base, dims)), p + n - pos
    names = {2: "time", 4: "bitfield", 5: "opaque", 7: "reference", 8: "enumerated", 9: "variable-length"}
    raise H5Error(f"{names.get(cls, f'class {cls}')} datatype")


def _dataspace(r: _Reader, pos: int) -> Optional[Tuple[int, ...]]:
    """Dimensions of a dataspace message (specification IV.A.2.b); None for a null one."""
    version, rank, flags = r.u(pos, 1), r.u(pos + 1, 1), r.u(pos + 2, 1)
    if version == 1:
        p = pos + 8
    elif version == 2:
        if r.u(pos + 3, 1) == 2:
            return None
        p = pos + 4
    else:
        raise H5Error(f"dataspace message version {version}")
    return tuple(r.length(p + i * r.sl) for i in range(rank))


# ---------------------------------------------------------------------------------------
# objects

def _header_messages(r: _Reader, addr: int) -> list:
    """Messages of the version 1 object header at addr, continuation blocks included."""
    if r.raw(addr, 4) == b"OHDR":
        raise H5Error("version 2 object header (a file written with the format's newer structures)")
    version, count, size = r.u(addr, 1), r.u(addr + 2, 2), r.u(addr + 8, 4)
    if version != 1:
        raise H5Error(f"object header version {version} at {addr}")
    blocks = [(addr + 16, size)]
    out = []
    while blocks:
        start, length = blocks.pop(0)
        p, end = start, start + length
        while p + 8 <= end and len(out) < count:
            mtype, msize, mflags = r.u(p, 2), r.u(p + 2, 2), r.u(p + 4, 1)
            data = p + 8
            if data + msize > end:
                raise H5Error(f"header message at {p} overruns its block")
            if mtype == _MSG_CONTINUATION:
                blocks.append((r.addr(data), r.length(data + r.so)))
            out.append(_Message(mtype, mflags, data, msize))
            p = data + msize
    return out


def _check_unshared(m: _Message, what: str):
    if m.flags & 0x02:
        raise H5Error(f"shared {what} message")


class _Object:
    def __init__(self, file: "File", addr: int, name: str):
        self.file = file
        self.addr = addr
        self.name = name
        self._messages = _header_messages(file._r, addr)

    def _first(self, mtype: int) -> Optional[_Message]:
        for m in self._messages:
            if m.type == mtype:
                return m
        return None

    @property
    def attrs(self) -> dict:
        """Attributes stored in the object header: name -> numpy scalar or array, or None
        for an attribute whose datatype this reader does not decode (variable-length
        strings, compounds, ...: Arepo's `Parameters` and `Config` groups may hold them)."""
        r = self.file._r
        out = {}
        if self._first(_MSG_ATTRIBUTE_INFO) is not None:
            # dense storage (fractal heap) holds no attributes when its address is undefined
            info = self._first(_MSG_ATTRIBUTE_INFO)
            flags = r.u(info.pos + 1, 1)
            heap = r.addr(info.pos + 2 + (2 if flags & 1 else 0))
            if heap is not None:
                raise H5Error(f"dense attribute storage on '{self.name}'")
        for m in self._messages:
            if m.type == _MSG_ATTRIBUTE:
                name, value = _attribute(r, m)
                out[name] = value
        return out


def _attribute(r: _Reader, m: _Message):
    """(name, value) of an attribute message (specification IV.A.2.m)."""
    version = r.u(m.pos, 1)
    flags = r.u(m.pos + 1, 1)
    nsize, tsize, ssize = r.u(m.pos + 2, 2), r.u(m.pos + 4, 2), r.u(m.pos + 6, 2)
    if version == 1:
        pad = lambda n: (n + 7) & ~7
        p = m.pos + 8
        name = r.raw(p, nsize).split(b"\0", 1)[0].decode("utf-8")
        p += pad(nsize)
        tpos = p
        p += pad(tsize)
        spos = p
        p += pad(ssize)
    elif version in (2, 3):
        if flags & 0x03:
            raise H5Error("attribute with a shared datatype or dataspace")
        p = m.pos + 8 + (1 if version == 3 else 0)
        name = r.raw(p, nsize).split(b"\0", 1)[0].decode("utf-8")
        tpos = p + nsize
        spos = tpos + tsize
        p = spos + ssize
    else:
        raise H5Error(f"attribute message version {version}")
    try:
        dtype = _datatype(r, tpos)
    except H5Error:
        return name, None
    shape = _dataspace(r, spos)
    if shape is None:
        return name, None
    n = int(np.prod(shape, dtype=np.int64)) if shape else 1
    data = np.frombuffer(r.raw(p, n * dtype.itemsize), dtype=dtype, count=n)
    value = data.reshape(tuple(shape) + dtype.shape) if shape else data[0]
    return name, value


class Group(_Object):
    """A group stored as a symbol table: its members by name."""

    def __init__(self, file: "File", addr: int, name: str):
        super().__init__(file, addr, name)
        st = self._first(_MSG_SYMBOL_TABLE)
        if st is None:
            if self._first(_MSG_LINK) is not None or self._first(_MSG_LINK_INFO) is not None:
                raise H5Error(f"group '{name}' stored with link messages (the format's newer groups)")
            raise H5Error(f"object '{name}' is not a group")
        r = file._r
        self._members = {}
        heap = r.addr(st.pos + r.so)
        if r.raw(heap, 4) != b"HEAP":
            raise H5Error(f"no local heap at {heap}")
        heap_data = r.addr(heap + 8 + 2 * r.sl)
        self._walk_group_tree(r, r.addr(st.pos), heap_data)

    def _walk_group_tree(self, r: _Reader, node: int, heap_data: int):
        if node is None:
            return
        if r.raw(node, 4) != b"TREE" or r.u(node + 4, 1) != 0:
            raise H5Error(f"no group B-tree node at {node}")
        level, used = r.u(node + 5, 1), r.u(node + 6, 2)
        p = node + 8 + 2 * r.so + r.sl  # first key, then child, key, child, ...
        for i in range(used):
            child = r.addr(p + i * (r.sl + r.so))
            if level > 0:
                self._walk_group_tree(r, child, heap_data)
                continue
            if r.raw(child, 4) != b"SNOD":
                raise H5Error(f"no symbol node at {child}")
            entry = child + 8
            for _ in range(r.u(child + 6, 2)):
                name = r.cstring(heap_data + r.u(entry, r.so))  # link name offset into the heap
                self._members[name] = r.addr(entry + r.so)
                entry += 2 * r.so + 24

    def keys(self):
        return list(self._members)

    def __contains__(self, path: str) -> bool:
        try:
            self[path]
        except KeyError:
            return False
        return True

    def __getitem__(self, path: str) -> Union["Group", "Dataset"]:
        head, _, rest = path.strip("/").partition("/")
        if head not in self._members:
            raise KeyError(f"no member '{head}' in group '{self.name}'")
        full = f"{self.name.rstrip('/')}/{head}"
        obj = self.file._open(self._members[head], full)
        if rest:
            if not isinstance(obj, Group):
                raise KeyError(f"'{full}' is not a group")
            return obj[rest]
        return obj


class Dataset(_Object):
    """A dataset: `shape`, `dtype`, `attrs`; `read()` returns the data as a numpy array."""

    def __init__(self, file: "File", addr: int, name: str):
        super().__init__(file, addr, name)
        r = file._r
        for mtype, what in ((_MSG_DATATYPE, "datatype"), (_MSG_DATASPACE, "dataspace")):
            m = self._first(mtype)
            if m is None:
                raise H5Error(f"dataset '{name}' has no {what} message")
            _check_unshared(m, what)
        self.dtype = _datatype(r, self._first(_MSG_DATATYPE).pos)
        shape = _dataspace(r, self._first(_MSG_DATASPACE).pos)
        self.shape = () if shape is None else shape
        self._null = shape is None
        self._layout = self._parse_layout(r)
        self._filters = self._parse_filters(r)

    def _parse_layout(self, r: _Reader):
        m = self._first(_MSG_LAYOUT)
        if m is None:
            raise H5Error(f"dataset '{self.name}' has no layout message")
        version, p = r.u(m.pos, 1), m.pos
        if version in (1, 2):
            ndim, cls = r.u(p + 1, 1), r.u(p + 2, 1)
            p += 8
            addr = None
            if cls in (1, 2):
                addr = r.addr(p)
                p += r.so
            dims = [r.u(p + 4 * i, 4) for i in range(ndim)]
            p += 4 * ndim
            if cls == 0:
                size = r.u(p, 4)
                return ("compact", p + 4, size)
            if cls == 1:
                return ("contiguous", addr, self._nbytes())
            elem = r.u(p, 4)
            return ("chunked", addr, tuple(dims[:-1]) if len(dims) == len(self.shape) + 1 else tuple(dims), elem)
        if version == 3:
            cls = r.u(p + 1, 1)
            if cls == 0:
                return ("compact", p + 4, r.u(p + 2, 2))
            if cls == 1:
                return ("contiguous", r.addr(p + 2), r.length(p + 2 + r.so))
            if cls == 2:
                ndim = r.u(p + 2, 1)
                addr = r.addr(p + 3)
                dims = [r.u(p + 3 + r.so + 4 * i, 4) for i in range(ndim)]
                return ("chunked", addr, tuple(dims[:-1]), dims[-1])
            raise H5Error(f"layout class {cls}")
        raise H5Error(f"data layout message version {version} (the format's newer chunk indexes)")

    def _parse_filters(self, r: _Reader):
        m = self._first(_MSG_FILTERS)
        if m is None:
            return []
        version, count = r.u(m.pos, 1), r.u(m.pos + 1, 1)
        p = m.pos + (8 if version == 1 else 2)
        out = []
        for _ in range(count):
            fid = r.u(p, 2)
            if version == 1 or fid >= 256:
                name_len = r.u(p + 2, 2)
                p += 4
            else:
                name_len = 0
                p += 2
            flags, nvals = r.u(p, 2), r.u(p + 2, 2)
            p += 4
            p += ((name_len + 7) & ~7) if version == 1 else name_len
            vals = [r.u(p + 4 * i, 4) for i in range(nvals)]
            p += 4 * nvals
            if version == 1 and nvals % 2:
                p += 4
            if fid not in (_FILTER_DEFLATE, _FILTER_SHUFFLE, _FILTER_FLETCHER32):
                raise H5Error(f"dataset '{self.name}' uses filter {fid} (only deflate, shuffle, fletcher32 are read)")
            out.append((fid, flags, vals))
        return out

    def _nbytes(self) -> int:
        return int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize

    def __len__(self) -> int:
        if not self.shape:
            raise TypeError("len() of a scalar dataset")
        return self.shape[0]

    def read(self, start: Optional[int] = None, stop: Optional[int] = None) -> np.ndarray:
        """Rows [start, stop) along the first axis (all of them by default), in native
        byte order; an array element type adds its dimensions as trailing axes, a
        compound one gives a structured array."""
        if self._null:
            return np.empty(0, self.dtype.newbyteorder("="))
        if not self.shape:
            out = self._read_rows(0, 1, scalar=True)
            return out.reshape(self.dtype.shape)
        n0 = self.shape[0]
        lo, hi, _ = slice(start, stop).indices(n0)
        hi = max(hi, lo)
        return self._read_rows(lo, hi)

    def _read_rows(self, lo: int, hi: int, scalar: bool = False) -> np.ndarray:
        r = self.file._r
        shape = (1,) if scalar else self.shape
        row = int(np.prod(shape[1:], dtype=np.int64))
        out_shape = (hi - lo,) + tuple(shape[1:])
        n = (hi - lo) * row
        kind = self._layout[0]
        if kind in ("compact", "contiguous"):
            addr = self._layout[1]
            if addr is None or n == 0:
                data = np.zeros(n, self.dtype)
            else:
                data = r.array(addr + lo * row * self.dtype.itemsize, self.dtype, n)
            out = data.reshape(out_shape + self.dtype.shape)  # an array type adds trailing axes
        else:
            out = self._read_chunked(r, lo, hi, shape, out_shape)
        return np.ascontiguousarray(out.astype(self.dtype.base.newbyteorder("="), copy=True))

    def _read_chunked(self, r: _Reader, lo: int, hi: int, shape, out_shape) -> np.ndarray:
        _, btree, chunk, elem = self._layout
        if elem != self.dtype.itemsize or len(chunk) != len(shape):
            raise H5Error(f"dataset '{self.name}': chunk dimensions {chunk} do not match {shape}")
        out = np.zeros(out_shape, self.dtype)
        if btree is None or out.size == 0:
            return out
        for offsets, size, mask, addr in self._chunks(r, btree, len(shape)):
            if offsets[0] >= hi or offsets[0] + chunk[0] <= lo:
                continue
            raw = r.raw(addr, size)
            for i, (fid, _, vals) in reversed(list(enumerate(self._filters))):
                if mask & (1 << i):
                    continue
                if fid == _FILTER_DEFLATE:
                    raw = zlib.decompress(raw)
                elif fid == _FILTER_SHUFFLE:
                    width = vals[0] if vals else elem
                    k = len(raw) // width
                    body = np.frombuffer(raw[:k * width], np.uint8).reshape(width, k).T.reshape(-1)
                    raw = body.tobytes() + raw[k * width:]
                else:  # Fletcher-32: a 4-byte checksum after the data
                    raw = raw[:-4]
            full = int(np.prod(chunk, dtype=np.int64))
            if len(raw) < full * elem:
                raise H5Error(f"dataset '{self.name}': chunk at {addr} holds {len(raw)} bytes, needs {full * elem}")
            block = np.frombuffer(raw, self.dtype, count=full).reshape(tuple(chunk) + self.dtype.shape)
            src, dst = [], []
            for axis, (o, c, s) in enumerate(zip(offsets, chunk, shape)):
                a, b = (max(o, lo), min(o + c, hi)) if axis == 0 else (o, min(o + c, s))
                src.append(slice(a - o, b - o))
                dst.append(slice(a - lo, b - lo) if axis == 0 else slice(a, b))
            out[tuple(dst)] = block[tuple(src)]
        return out

    def _chunks(self, r: _Reader, node: int, rank: int):
        """(offsets, stored size, filter mask, address) of every chunk under a type 1
        B-tree node."""
        if r.raw(node, 4) != b"TREE" or r.u(node + 4, 1) != 1:
            raise H5Error(f"no chunk B-tree node at {node}")
        level, used = r.u(node + 5, 1), r.u(node + 6, 2)
        key = 8 + 8 * (rank + 1)
        p = node + 8 + 2 * r.so
        for i in range(used):
            k = p + i * (key + r.so)
            child = r.addr(k + key)
            if level > 0:
                yield from self._chunks(r, child, rank)
                continue
            size, mask = r.u(k, 4), r.u(k + 4, 4)
            offsets = tuple(r.u(k + 8 + 8 * j, 8) for j in range(rank))
            yield offsets, size, mask, child


class File:
    """An HDF5 file opened for reading (memory-mapped): `f["PartType0/Masses"].read()`,
    `f.attrs`, `f.keys()`.  Use as a context manager or call close()."""

    def __init__(self, path: Union[str, os.PathLike]):
        self.path = pathlib.Path(path)
        self._fh = open(self.path, "rb")
        try:
            size = os.fstat(self._fh.fileno()).st_size
            self._buf = mmap.mmap(self._fh.fileno(), 0, access=mmap.ACCESS_READ) if size else b""
            base = self._find_superblock(size)
            self._r = self._parse_superblock(base)
            self._objects = {}
            self.root = Group(self, self._root_addr, "/")
        except Exception:
            self.close()
            raise

    def _find_superblock(self, size: int) -> int:
        pos = 0
        while pos + 8 <= size:
            if self._buf[pos:pos + 8] == SIGNATURE:
                return pos
            pos = 512 if pos == 0 else 2 * pos
        raise H5Error(f"{self.path}: not an HDF5 file")

    def _parse_superblock(self, at: int) -> _Reader:
        b = self._buf
        version = b[at + 8]
        if version not in (0, 1):
            raise H5Error(f"{self.path}: superblock version {version} (the format's newer structures)")
        so, sl = b[at + 13], b[at + 14]
        if so not in (2, 4, 8) or sl not in (2, 4, 8):
            raise H5Error(f"{self.path}: offsets of {so} and lengths of {sl} bytes")
        p = at + 24 + (4 if version == 1 else 0)
        base = int.from_bytes(b[p:p + so], "little")
        r = _Reader(b, base, so, sl)
        entry = p + 4 * so  # base, free space, end of file, driver info; then the root entry
        self._root_addr = r.addr(entry + so)
        return r

    def _open(self, addr: int, name: str):
        obj = self._objects.get(addr)
        if obj is None:
            msgs = _header_messages(self._r, addr)
            types = {m.type for m in msgs}
            if _MSG_LAYOUT in types:
                obj = Dataset(self, addr, name)
            else:
                obj = Group(self, addr, name)
            self._objects[addr] = obj
        return obj

    def __getitem__(self, path: str):
        return self.root[path]

    def __contains__(self, path: str) -> bool:
        return path in self.root

    def keys(self):
        return self.root.keys()

    @property
    def attrs(self) -> dict:
        return self.root.attrs

    def close(self):
        buf = getattr(self, "_buf", None)
        if isinstance(buf, mmap.mmap):
            buf.close()
        self._buf = b""
        if getattr(self, "_fh", None) is not None:
            self._fh.close()
            self._fh = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


# ---------------------------------------------------------------------------------------
# datasets with units, as the reference reads them

@dataclasses.dataclass(frozen=True)
class Dimension:
    """Exponents of a quantity's unit (src/units/dimension.rs): SI base units, plus the
    cosmological scale factor a and the Hubble parameter h."""
    length: int = 0
    time: int = 0
    mass: int = 0
    temperature: int = 0
    h: int = 0
    a: int = 0

    def non_cosmological(self) -> "Dimension":
        return dataclasses.replace(self, h=0, a=0)


NONE = Dimension()
LENGTH = Dimension(length=1)
AREA = Dimension(length=2)
MASS = Dimension(mass=1)
TEMPERATURE = Dimension(temperature=1)
DENSITY = Dimension(length=-3, mass=1)
ENERGY_PER_MASS = Dimension(length=2, time=-2)


def _scalar_float(value, name: str, dataset: str) -> float:
    if value is None or np.ndim(value) != 0 or np.asarray(value).dtype.kind not in "iuf":
        raise H5Error(f"attribute '{name}' of dataset '{dataset}' is not a number")
    return float(value)


def _scalar_int(value, name: str, dataset: str) -> int:
    """An integer attribute read as the library converts it to i32 (truncation)."""
    return int(_scalar_float(value, name, dataset))


class DefaultUnits:
    """The reference's own dataset attributes (src/io/unit_reader.rs:37-67): the SI scale
    factor `scale_factor_si` and integer exponents `scaling_length`, `scaling_mass`,
    `scaling_time`, `scaling_temperature`."""

    def scale_factor(self, ds: Dataset) -> float:
        attrs = ds.attrs
        if "scale_factor_si" not in attrs:
            raise H5Error("No scale factor in dataset")
        return _scalar_float(attrs["scale_factor_si"], "scale_factor_si", ds.name)

    def dimension(self, ds: Dataset) -> Dimension:
        attrs = ds.attrs
        got = {}
        for key, field, what in (("scaling_length", "length", "length"), ("scaling_mass", "mass", "mass"),
                                 ("scaling_time", "time", "time"),
                                 ("scaling_temperature", "temperature", "temperature")):
            if key not in attrs:
                raise H5Error(f"No {what} scale factor in dataset")
            got[field] = _scalar_int(attrs[key], key, ds.name)
        return Dimension(**got)


class IdUnits:
    """Identifiers and flags: factor 1, dimensionless (src/io/unit_reader.rs:69-80)."""

    def scale_factor(self, ds: Dataset) -> float:
        return 1.0

    def dimension(self, ds: Dataset) -> Dimension:
        return NONE


class ArepoUnits:
    """Arepo's dataset attributes (src/arepo_postprocess/unit_reader.rs:45-128): `to_cgs`
    and the exponents `length_scaling`, `mass_scaling`, `velocity_scaling`, `a_scaling`,
    `h_scaling`.  Length exponent = length + velocity, time exponent = -velocity; the
    factor is (1 / cosmology factor if a or h appear) * 0.01^length * 0.001^mass * to_cgs,
    and a `to_cgs` of 0 means 1 for a dimensionless dataset."""

    def __init__(self, cosmology: Optional[Cosmology] = None):
        self.cosmology = cosmology

    def _raw_dimension(self, ds: Dataset) -> Dimension:
        attrs = ds.attrs
        got = {}
        for key, what in (("length_scaling", "length scale factor"), ("mass_scaling", "mass scale factor"),
                          ("velocity_scaling", "velocity scale factor"), ("a_scaling", "a scale factor"),
                          ("h_scaling", "h scale factor")):
            if key not in attrs:
                raise H5Error(f"No {what} in dataset: '{ds.name}'")
            got[key] = _scalar_int(attrs[key], key, ds.name)
        return Dimension(length=got["length_scaling"] + got["velocity_scaling"], mass=got["mass_scaling"],
                         time=-got["velocity_scaling"], temperature=0, h=got["h_scaling"], a=got["a_scaling"])

    def _check_cosmology(self):
        if self.cosmology is None:
            raise H5Error("Cosmological units in input file, but no cosmology given. "
                          "Add cosmology section to parameter file?")

    def scale_factor(self, ds: Dataset) -> float:
        d = self._raw_dimension(ds)
        cosmological = d.a != 0 or d.h != 0
        if cosmological:
            self._check_cosmology()
            cosmo = 1.0 / self.cosmology.factor(d)
        else:
            cosmo = 1.0
        cgs_to_si = 0.01 ** d.length * 0.001 ** d.mass
        attrs = ds.attrs
        if "to_cgs" not in attrs:
            raise H5Error("No scale factor in dataset")
        cgs = _scalar_float(attrs["to_cgs"], "to_cgs", ds.name)
        if cgs == 0.0:
            if d != NONE:
                raise H5Error(f"unit scale factor 0 in dataset '{ds.name}' of dimension {d}")
            cgs = 1.0
        return cosmo * cgs_to_si * cgs

    def dimension(self, ds: Dataset) -> Dimension:
        d = self._raw_dimension(ds)
        if d.a == 0 and d.h == 0:
            return d
        self._check_cosmology()
        return d.non_cosmological()


def input_files(path: Union[str, os.PathLike]) -> list:
    """The file itself, or every `*.hdf5` file in a directory
    (src/io/input/mod.rs:75-97 `get_file_or_all_hdf5_files_in_path_if_dir`).  The
    reference takes the directory's listing order, which the OS leaves unspecified;
    here the files are sorted by name."""
    p = pathlib.Path(path)
    if p.is_file():
        return [p]
    if not p.is_dir():
        raise H5Error(f"Failed to open file: {p}")
    return sorted(q for q in p.iterdir() if q.is_file() and q.suffix == ".hdf5")


def read_dataset(paths: Union[str, os.PathLike, Sequence], name: str, dimension: Dimension,
                 units=None) -> np.ndarray:
    """Dataset `name` of every input file, concatenated in file order, in SI units.

    Restates the single-rank `Reader::full(..).read_dataset` (src/io/input/mod.rs:232-299):
    a file without the dataset contributes no rows; each file's values are multiplied by
    (the file's scale factor / the base conversion factor, 1 for SI); a dataset whose
    stored dimension differs from `dimension` is an error, "Mismatch in dimension while
    reading dataset {name}."  `units` is DefaultUnits() (the default), IdUnits() or
    ArepoUnits(cosmology).  Integer datasets with a factor of 1 keep their type."""
    units = DefaultUnits() if units is None else units
    if isinstance(paths, (str, os.PathLike)):
        paths = [paths]
    files = [f for p in paths for f in input_files(p)]
    parts = []
    for path in files:
        with File(path) as f:
            if name not in f:
                continue  # the reference warns of an empty dataset and reads 0 rows
            ds = f[name]
            if not isinstance(ds, Dataset):
                raise H5Error(f"Failed to open dataset: {name}")
            factor_written = units.scale_factor(ds)
            if units.dimension(ds) != dimension:
                raise H5Error(f"Mismatch in dimension while reading dataset {name}.")
            data = ds.read()
            if data.dtype.names:
                # a vector stored as a compound of numbers ({x, y, z}): its fields on a
                # trailing axis, like a vector stored as an array type
                if any(data.dtype[n].kind not in "iuf" or data.dtype[n].shape for n in data.dtype.names):
                    raise H5Error(f"dataset {name}: compound members are not all numbers")
                data = np.stack([data[n] for n in data.dtype.names], axis=-1)
            factor = factor_written / 1.0  # factor_written / base_conversion_factor (SI: 1)
            if factor != 1.0 or data.dtype.kind == "f":
                data = data.astype(np.float64) * factor
            parts.append(data)
    if not parts:
        return np.empty(0)
    return np.concatenate(parts)
