"""HDF5 files without h5py: the subset of the format that h5py and libhdf5
write by default, read and written in numpy.

gala serialises orbits, phase-space positions and mock streams through h5py
(``Orbit.to_hdf5`` / ``from_hdf5``, src/gala/dynamics/orbit.py:236-323;
``PhaseSpacePosition.to_hdf5``, src/gala/dynamics/core.py:572-640;
``MockStream.to_hdf5``, src/gala/dynamics/mockstream/core.py:106-150; the
quantity helpers in src/gala/io.py:4-47).  Neither h5py nor libhdf5 is part of
this library's dependencies, so this module implements the pieces of the HDF5
file format (The HDF Group, "HDF5 File Format Specification", version 2) that
those files use, with an interface shaped like h5py's:

* superblock version 0 (version 1 is read too), 8-byte offsets and lengths;
* version-1 object headers with continuation blocks;
* "old-style" groups: a symbol-table message pointing at a version-1 B-tree of
  symbol-table nodes (SNOD) and a local heap of link names;
* datasets with a version-1/2 dataspace (scalar or simple), a fill-value
  message and a version-3 layout message (contiguous or compact; chunked
  layouts with deflate and shuffle filters are read as the specification
  describes them, untested: no chunked file written by libhdf5 was at hand);
* datatypes: IEEE floats, integers, fixed-length strings and variable-length
  strings (stored in global heap collections);
* version-1 attribute messages (versions 2 and 3 are read too).

Writing builds the whole tree in memory and lays the file out on ``close()``,
the way h5py's default (``libver='earliest'``) files look: the same object
kinds, node sizes (group leaf node K = 4, group internal node K = 16) and
message encodings, so libhdf5 reads what is written here and this module reads
what h5py writes.  Groups written here hold at most 2 x 4 = 8 links per
symbol-table node and up to 32 nodes (256 links) per group.
"""
from __future__ import annotations

import struct
import zlib
from collections import OrderedDict

import numpy as np

__all__ = ["File", "Group", "Dataset", "string_dtype"]

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF
_LEAF_K = 4        # symbol-table node: up to 2K entries
_INTERNAL_K = 16   # group B-tree node: up to 2K children
_ENTRY = 40        # symbol-table entry size with 8-byte offsets
_SNOD_SIZE = 8 + 2 * _LEAF_K * _ENTRY
_TREE_SIZE = 24 + (2 * _INTERNAL_K + 1) * 8 + 2 * _INTERNAL_K * 8
_GCOL_MIN = 4096


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ============================================================================
# datatypes
# ============================================================================
class _VlenStr:
    """Marker dtype for variable-length strings (h5py's ``string_dtype()``)."""

    def __init__(self, encoding="utf-8"):
        self.encoding = encoding

    def __repr__(self):
        return f"string_dtype({self.encoding!r})"

    def __eq__(self, other):
        return isinstance(other, _VlenStr) and other.encoding == self.encoding

    def __hash__(self):
        return hash(("vlen", self.encoding))


def string_dtype(encoding="utf-8", length=None):
    """Variable-length (length None) or fixed-length string type, as in h5py."""
    if length is None:
        return _VlenStr(encoding)
    return np.dtype(f"S{int(length)}")


def _encode_dtype(dt) -> bytes:
    """Datatype message (class and version, bit fields, size, properties)."""
    if isinstance(dt, _VlenStr):
        cset = 1 if dt.encoding.lower().replace("-", "") == "utf8" else 0
        base = _encode_dtype(np.dtype("u1"))
        return bytes([0x19, 0x01, cset, 0x00]) + struct.pack("<I", 16) + base
    dt = np.dtype(dt)
    if dt.kind == "f":
        if dt.itemsize == 8:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            sign = 63
        elif dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            sign = 31
        else:
            raise TypeError(f"unsupported float type {dt}")
        order = 1 if dt.byteorder == ">" else 0
        return bytes([0x11, 0x20 | order, sign, 0x00]) + struct.pack("<I", dt.itemsize) + props
    if dt.kind in "iu":
        flags = (0x08 if dt.kind == "i" else 0) | (1 if dt.byteorder == ">" else 0)
        return bytes([0x10, flags, 0, 0]) + struct.pack("<I", dt.itemsize) + struct.pack("<HH", 0, 8 * dt.itemsize)
    if dt.kind == "S":
        # null-padded ASCII, as h5py stores numpy bytes arrays
        return bytes([0x13, 0x01, 0x00, 0x00]) + struct.pack("<I", max(dt.itemsize, 1))
    raise TypeError(f"unsupported datatype {dt}")


def _decode_dtype(buf: bytes, p: int):
    """Returns (dtype or _VlenStr or a description tuple, bytes consumed)."""
    cv = buf[p]
    cls, ver = cv & 0x0F, cv >> 4
    b0, b1, b2 = buf[p + 1], buf[p + 2], buf[p + 3]
    size = struct.unpack_from("<I", buf, p + 4)[0]
    q = p + 8
    if cls == 0:  # fixed-point
        order = ">" if b0 & 1 else "<"
        signed = bool(b0 & 0x08)
        return np.dtype(f"{order}{'i' if signed else 'u'}{size}"), 8 + 4
    if cls == 1:  # floating point
        order = ">" if b0 & 1 else "<"
        return np.dtype(f"{order}f{size}"), 8 + 12
    if cls == 3:  # fixed-length string
        return np.dtype(f"S{size}"), 8
    if cls == 9:  # variable length
        base, nb = _decode_dtype(buf, q)
        if (b0 & 0x0F) == 1:
            return _VlenStr("utf-8" if (b1 & 0x0F) == 1 else "ascii"), 8 + nb
        return ("vlen", base), 8 + nb
    if cls == 6:  # compound (read as a numpy structured type)
        nmemb = b0 | (b1 << 8)
        names, formats, offsets = [], [], []
        for _ in range(nmemb):
            end = buf.index(b"\x00", q)
            name = buf[q:end].decode()
            if ver < 3:
                q = q + _pad8(end - q + 1)
            else:
                q = end + 1
            if ver == 3:
                nbytes = max(1, (size.bit_length() + 7) // 8)
                off = int.from_bytes(buf[q:q + nbytes], "little")
                q += nbytes
            else:
                off = struct.unpack_from("<I", buf, q)[0]
                q += 4
                if ver == 1:
                    q += 1 + 3 + 4 + 4 + 16  # dimensionality, reserved, permutation, reserved, 4 dims
            mdt, nb = _decode_dtype(buf, q)
            q += nb
            names.append(name)
            formats.append(mdt)
            offsets.append(off)
        return np.dtype({"names": names, "formats": formats, "offsets": offsets, "itemsize": size}), q - p
    if cls == 8:  # enumeration (h5py bool): read as the base integer type
        base, nb = _decode_dtype(buf, q)
        nmemb = b0 | (b1 << 8)
        q2 = q + nb
        for _ in range(nmemb):
            end = buf.index(b"\x00", q2)
            q2 = q2 + (_pad8(end - q2 + 1) if ver < 3 else end - q2 + 1)
        q2 += nmemb * base.itemsize
        return base, q2 - p
    raise NotImplementedError(f"HDF5 datatype class {cls} is not supported")


def _dtype_size(dt) -> int:
    return 16 if isinstance(dt, _VlenStr) else np.dtype(dt).itemsize


# ============================================================================
# dataspace
# ============================================================================
def _encode_space(shape) -> bytes:
    """Version-1 dataspace; a simple one carries its maximum dimensions (equal
    to the dimensions), as libhdf5 writes it."""
    shape = tuple(int(s) for s in shape)
    out = bytes([1, len(shape), 1 if shape else 0, 0]) + b"\x00" * 4
    out += b"".join(struct.pack("<Q", s) for s in shape) * (2 if shape else 0)
    return out


def _decode_space(buf: bytes, p: int):
    ver, rank, flags = buf[p], buf[p + 1], buf[p + 2]
    if ver == 1:
        q = p + 8
    elif ver == 2:
        if buf[p + 3] == 2:  # null dataspace
            return None
        q = p + 4
    else:
        raise NotImplementedError(f"dataspace version {ver}")
    return tuple(struct.unpack_from(f"<{rank}Q", buf, q)) if rank else ()


# ============================================================================
# reading
# ============================================================================
class _Reader:
    def __init__(self, data: bytes):
        self.b = data
        self._gcol = {}
        if data[:8] != _SIG:
            raise OSError("not an HDF5 file (signature not found at offset 0)")
        ver = data[8]
        if ver not in (0, 1):
            raise NotImplementedError(f"HDF5 superblock version {ver} (files written with libver='latest')")
        if data[13] != 8 or data[14] != 8:
            raise NotImplementedError("only 8-byte offsets and lengths are supported")
        p = 24 + (4 if ver == 1 else 0)
        self.base = struct.unpack_from("<Q", data, p)[0]
        root_entry = p + 32
        self.root_header = struct.unpack_from("<Q", data, root_entry + 8)[0]

    def u(self, fmt, p):
        return struct.unpack_from(fmt, self.b, p)

    # --- object headers -----------------------------------------------------
    def messages(self, addr):
        """[(type, flags, bytes)] of the version-1 object header at addr."""
        b = self.b
        if b[addr:addr + 4] == b"OHDR":
            raise NotImplementedError("version-2 object headers (libver='latest') are not supported")
        ver, _, nmsg, _, size = self.u("<BBHII", addr)
        if ver != 1:
            raise OSError(f"bad object header version {ver} at {addr}")
        out = []
        blocks = [(addr + 16, size)]
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p + 8 <= end and len(out) < nmsg:
                mtype, msize, mflags = self.u("<HHB", p)
                body = b[p + 8:p + 8 + msize]
                out.append((mtype, mflags, body))
                if mtype == 0x10:
                    blocks.append(struct.unpack_from("<QQ", body, 0))
                p += 8 + msize
        return out

    # --- heaps ------------------------------------------------------------------
    def local_heap(self, addr):
        if self.b[addr:addr + 4] != b"HEAP":
            raise OSError("local heap signature not found")
        size, _free, data = self.u("<QQQ", addr + 8)
        return self.b[data:data + size]

    def gheap_object(self, addr, index):
        col = self._gcol.get(addr)
        if col is None:
            if self.b[addr:addr + 4] != b"GCOL":
                raise OSError("global heap signature not found")
            csize = self.u("<Q", addr + 8)[0]
            col, p, end = {}, addr + 16, addr + csize
            while p + 16 <= end:
                idx, _nref, _, osize = self.u("<HHIQ", p)
                if idx == 0:
                    break
                col[idx] = self.b[p + 16:p + 16 + osize]
                p += 16 + _pad8(osize)
            self._gcol[addr] = col
        return col[index]

    def vlen_strings(self, raw: bytes, n: int, enc: str):
        out = []
        for k in range(n):
            length, addr, idx = struct.unpack_from("<IQI", raw, 16 * k)
            if length == 0 or addr in (0, _UNDEF):
                s = b""
            else:
                s = self.gheap_object(addr, idx)[:length]
            out.append(s.decode(enc) if enc == "utf-8" else s)
        return out

    # --- groups -----------------------------------------------------------------
    def group_links(self, msgs):
        """OrderedDict name -> object header address, in name order."""
        links = OrderedDict()
        for mtype, _, body in msgs:
            if mtype == 0x11:
                btree, heap = struct.unpack_from("<QQ", body, 0)
                names = self.local_heap(heap)
                self._walk_group_btree(btree, names, links)
            elif mtype == 0x06:  # link message (new-style compact group)
                name, addr = self._link_message(body)
                if addr is not None:
                    links[name] = addr
        return links

    def _link_message(self, body):
        ver, flags = body[0], body[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = body[p]
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nsz = 1 << (flags & 3)
        nlen = int.from_bytes(body[p:p + nsz], "little")
        p += nsz
        name = body[p:p + nlen].decode()
        p += nlen
        if ltype != 0:
            return name, None
        return name, struct.unpack_from("<Q", body, p)[0]

    def _walk_group_btree(self, addr, names, links):
        b = self.b
        if b[addr:addr + 4] != b"TREE":
            raise OSError("v1 B-tree signature not found")
        ntype, level, used = self.u("<BBH", addr + 4)
        p = addr + 24
        children = [self.u("<Q", p + 8 + 16 * i)[0] for i in range(used)]
        for c in children:
            if level > 0:
                self._walk_group_btree(c, names, links)
                continue
            if b[c:c + 4] != b"SNOD":
                raise OSError("symbol table node signature not found")
            nsym = self.u("<H", c + 6)[0]
            for k in range(nsym):
                e = c + 8 + _ENTRY * k
                name_off, header = self.u("<QQ", e)
                end = names.index(b"\x00", name_off)
                links[names[name_off:end].decode()] = header

    # --- datasets and attributes ----------------------------------------------
    def read_raw(self, msgs, dt, shape):
        layout = next((body for t, _, body in msgs if t == 0x08), None)
        filters = next((body for t, _, body in msgs if t == 0x0B), None)
        n = int(np.prod(shape)) if shape is not None else 0
        nbytes = n * _dtype_size(dt)
        if layout is None:
            raise OSError("dataset without a layout message")
        ver = layout[0]
        if ver != 3:
            raise NotImplementedError(f"layout message version {ver}")
        cls = layout[1]
        if cls == 0:
            size = struct.unpack_from("<H", layout, 2)[0]
            return layout[4:4 + size]
        if cls == 1:
            addr, size = struct.unpack_from("<QQ", layout, 2)
            if addr == _UNDEF:
                return b"\x00" * nbytes
            return memoryview(self.b)[addr:addr + size]
        if cls == 2:
            return self._read_chunked(layout, filters, dt, shape)
        raise NotImplementedError(f"layout class {cls}")

    def _read_chunked(self, layout, filters, dt, shape):
        rank = layout[2]  # dimensionality + 1 (the last is the element size)
        btree = struct.unpack_from("<Q", layout, 3)[0]
        cdims = struct.unpack_from(f"<{rank}I", layout, 11)
        chunk = tuple(cdims[:-1])
        esize = cdims[-1]
        pipeline = []  # filter ids in the order they were applied on writing
        if filters is not None:
            fver, nf = filters[0], filters[1]
            q = 8 if fver == 1 else 2
            for _ in range(nf):
                fid = struct.unpack_from("<H", filters, q)[0]
                named = fver == 1 or fid >= 256
                namelen = struct.unpack_from("<H", filters, q + 2)[0] if named else 0
                _flags, ncv = struct.unpack_from("<HH", filters, q + 4 if named else q + 2)
                q += (8 if named else 6) + (_pad8(namelen) if fver == 1 else namelen) + 4 * ncv
                if fver == 1 and ncv % 2:
                    q += 4
                if fid not in (1, 2):  # deflate, shuffle
                    raise NotImplementedError(f"HDF5 filter {fid}")
                pipeline.append(fid)
        out = np.zeros(int(np.prod(shape)) * esize, dtype=np.uint8).reshape(tuple(shape) + (esize,))
        nchunk = int(np.prod(chunk))
        for offs, fmask, raw in self._chunks(btree, rank):
            data = raw
            # undo the filters in reverse; bit k of the mask marks filter k as skipped
            for k in reversed(range(len(pipeline))):
                if fmask & (1 << k):
                    continue
                if pipeline[k] == 1:
                    data = zlib.decompress(data)
                elif esize > 1:
                    arr = np.frombuffer(data, dtype=np.uint8)
                    body = arr[:nchunk * esize].reshape(esize, nchunk).T.ravel()
                    data = body.tobytes() + arr[nchunk * esize:].tobytes()
            arr = np.frombuffer(data, dtype=np.uint8)[:nchunk * esize].reshape(chunk + (esize,))
            sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, chunk, shape))
            out[sl] = arr[tuple(slice(0, s.stop - s.start) for s in sl)]
        return out.tobytes()

    def _chunks(self, addr, rank):
        b = self.b
        if b[addr:addr + 4] != b"TREE":
            raise OSError("chunk B-tree signature not found")
        _, level, used = self.u("<BBH", addr + 4)
        ksize = 8 + 8 * rank
        p = addr + 24
        for i in range(used):
            key = p + i * (ksize + 8)
            csize, fmask = self.u("<II", key)
            offs = self.u(f"<{rank}Q", key + 8)[:-1]
            child = self.u("<Q", key + ksize)[0]
            if level > 0:
                yield from self._chunks(child, rank)
            else:
                yield offs, fmask, b[child:child + csize]

    def to_array(self, raw, dt, shape):
        if shape is None:
            return np.zeros(0, dtype=np.float64)
        n = int(np.prod(shape)) if shape else 1
        if isinstance(dt, _VlenStr):
            vals = self.vlen_strings(raw, n, dt.encoding)
            arr = np.empty(n, dtype=object)
            arr[:] = vals
            return arr.reshape(shape) if shape else arr[0]
        if isinstance(dt, tuple):
            raise NotImplementedError("variable-length sequences are not supported")
        arr = np.frombuffer(raw[:n * dt.itemsize], dtype=dt).reshape(shape)
        if dt.byteorder == ">":
            arr = arr.astype(dt.newbyteorder("<"))
        return arr.copy() if shape else arr[()]

    def attributes(self, msgs):
        out = OrderedDict()
        for mtype, _, body in msgs:
            if mtype != 0x0C:
                continue
            ver = body[0]
            nlen, tlen, slen = struct.unpack_from("<HHH", body, 2)
            p = 8 + (1 if ver == 3 else 0)
            name = body[p:p + nlen - 1].decode()
            p += _pad8(nlen) if ver == 1 else nlen
            dt, _ = _decode_dtype(body, p)
            p += _pad8(tlen) if ver == 1 else tlen
            shape = _decode_space(body, p)
            p += _pad8(slen) if ver == 1 else slen
            out[name] = self.to_array(body[p:], dt, shape)
        return out


# ============================================================================
# the h5py-shaped objects
# ============================================================================
class AttributeManager:
    """``obj.attrs``: an ordered mapping of small arrays and strings."""

    def __init__(self, node):
        self._node = node

    def __getitem__(self, name):
        return self._node._attrs[name]

    def __setitem__(self, name, value):
        self._node._file._check_writable()
        self._node._attrs[name] = _as_storable(value)[0]

    def __contains__(self, name):
        return name in self._node._attrs

    def __iter__(self):
        return iter(self._node._attrs)

    def keys(self):
        return self._node._attrs.keys()

    def items(self):
        return self._node._attrs.items()

    def get(self, name, default=None):
        return self._node._attrs.get(name, default)

    def __len__(self):
        return len(self._node._attrs)


def _as_storable(value, dtype=None):
    """(numpy value, HDF5 type) for data given to a dataset or attribute, with
    h5py's conversions: str -> variable-length UTF-8 string, bytes ->
    variable-length ASCII string, sequences of either likewise, numbers and
    numeric arrays unchanged."""
    if isinstance(dtype, _VlenStr):
        arr = np.asarray(value, dtype=object)
        return arr, dtype
    if isinstance(value, str):
        return np.asarray(value, dtype=object), _VlenStr("utf-8")
    if isinstance(value, bytes):
        return np.asarray(value, dtype=object), _VlenStr("ascii")
    if isinstance(value, (list, tuple)) and value and all(isinstance(v, (str, bytes)) for v in value):
        enc = "utf-8" if isinstance(value[0], str) else "ascii"
        arr = np.empty(len(value), dtype=object)
        arr[:] = list(value)
        return arr, _VlenStr(enc)
    arr = np.asarray(value) if dtype is None else np.asarray(value, dtype=dtype)
    if arr.dtype.kind == "U":
        obj = np.empty(arr.shape, dtype=object)
        obj[...] = arr
        return obj, _VlenStr("utf-8")
    if arr.dtype.kind == "O":
        flat = arr.ravel()
        if flat.size and all(isinstance(v, str) for v in flat):
            return arr, _VlenStr("utf-8")
        if flat.size and all(isinstance(v, bytes) for v in flat):
            return arr, _VlenStr("ascii")
        raise TypeError("object arrays must hold only str or only bytes")
    if arr.dtype.kind == "b":
        raise TypeError("boolean data is not supported (h5py stores it as an enumeration)")
    if arr.dtype.kind not in "fiuS":
        raise TypeError(f"unsupported data type {arr.dtype}")
    if arr.dtype.byteorder == ">":
        arr = arr.astype(arr.dtype.newbyteorder("<"))
    return arr, arr.dtype


class _Node:
    def __init__(self, file, name):
        self._file = file
        self.name = name
        self._attrs = OrderedDict()

    @property
    def attrs(self):
        return AttributeManager(self)

    @property
    def file(self):
        return self._file


class Dataset(_Node):
    """A dataset: ``ds[()]`` / ``ds[:]`` / ``ds[...]`` return numpy data
    (variable-length strings as ``str`` for UTF-8 and ``bytes`` for ASCII)."""

    def __init__(self, file, name, data, dtype):
        super().__init__(file, name)
        self._data = data
        self.dtype = dtype

    @property
    def shape(self):
        return np.shape(self._data)

    @property
    def ndim(self):
        return len(self.shape)

    @property
    def size(self):
        return int(np.prod(self.shape))

    def __len__(self):
        if not self.shape:
            raise TypeError("len() of a scalar dataset")
        return self.shape[0]

    def __getitem__(self, key):
        d = self._data
        if key == () or key is Ellipsis:
            if isinstance(d, np.ndarray) and d.ndim == 0:
                return d[()]
            return d.copy() if isinstance(d, np.ndarray) else d
        return d[key]

    def __array__(self, dtype=None, copy=None):
        a = np.asarray(self._data)
        return a if dtype is None else a.astype(dtype)

    def __iter__(self):
        return iter(self[()])

    def __repr__(self):
        return f'<HDF5 dataset "{self.name.rsplit("/", 1)[-1]}": shape {self.shape}, type {self.dtype!r}>'


class Group(_Node):
    """A group: a mapping of names to groups and datasets; ``g["a/b"]`` walks
    paths."""

    def __init__(self, file, name):
        super().__init__(file, name)
        self._links = OrderedDict()

    def _child_name(self, key):
        return (self.name.rstrip("/") + "/" + key) if self.name != "/" else "/" + key

    def _resolve(self, path, create=False):
        node = self
        parts = [p for p in path.split("/") if p]
        if path.startswith("/"):
            node = self._file
        for i, part in enumerate(parts[:-1]):
            nxt = node._links.get(part)
            if nxt is None:
                if not create:
                    raise KeyError(f"Unable to open object (component '{part}' not found)")
                nxt = node.create_group(part)
            if not isinstance(nxt, Group):
                raise KeyError(f"'{part}' is not a group")
            node = nxt
        return node, parts[-1] if parts else ""

    def __getitem__(self, path):
        node, last = self._resolve(path)
        if last == "":
            return node
        try:
            return node._links[last]
        except KeyError:
            raise KeyError(f"Unable to open object (object '{last}' doesn't exist)") from None

    def __contains__(self, path):
        try:
            self[path]
            return True
        except KeyError:
            return False

    def get(self, path, default=None):
        try:
            return self[path]
        except KeyError:
            return default

    def __iter__(self):
        return iter(self._links)

    def __len__(self):
        return len(self._links)

    def keys(self):
        return self._links.keys()

    def values(self):
        return self._links.values()

    def items(self):
        return self._links.items()

    def create_group(self, path):
        self._file._check_writable()
        node, last = self._resolve(path, create=True)
        if last in node._links:
            raise ValueError(f"Unable to create group (name already exists): {last}")
        g = Group(self._file, node._child_name(last))
        node._links[last] = g
        return g

    def require_group(self, path):
        return self[path] if path in self else self.create_group(path)

    def create_dataset(self, path, shape=None, dtype=None, data=None):
        self._file._check_writable()
        node, last = self._resolve(path, create=True)
        if last in node._links:
            raise ValueError(f"Unable to create dataset (name already exists): {last}")
        if data is None:
            if shape is None:
                raise TypeError("create_dataset needs data or a shape")
            data = np.zeros(shape, dtype=np.float64 if dtype is None else dtype)
        arr, dt = _as_storable(data, dtype)
        if shape is not None and tuple(np.shape(arr)) != tuple(shape):
            arr = np.reshape(arr, shape)
        ds = Dataset(self._file, node._child_name(last), arr, dt)
        node._links[last] = ds
        return ds

    def __setitem__(self, path, value):
        if isinstance(value, (Group, Dataset)):
            raise TypeError("hard links to existing objects are not supported")
        self.create_dataset(path, data=value)

    def __delitem__(self, path):
        self._file._check_writable()
        node, last = self._resolve(path)
        del node._links[last]

    def __repr__(self):
        return f'<HDF5 group "{self.name}" ({len(self)} members)>'


class File(Group):
    """An HDF5 file opened for reading ('r') or created for writing ('w', or
    'x' / 'w-' to refuse an existing file).  Written files are laid out and
    saved by ``close()`` (or at the end of a ``with`` block)."""

    def __init__(self, name, mode="r"):
        super().__init__(self, "/")
        self.filename = str(name)
        self.mode = mode
        self._closed = False
        if mode == "r":
            import mmap

            with open(self.filename, "rb") as fh:
                size = fh.seek(0, 2)
                if size < len(_SIG):
                    raise OSError("not an HDF5 file (signature not found at offset 0)")
                # mapped, not read: each dataset is copied once, straight from the map
                data = mmap.mmap(fh.fileno(), 0, access=mmap.ACCESS_READ)
            self._load(data)
        elif mode in ("w", "x", "w-"):
            if mode in ("x", "w-"):
                import os

                if os.path.exists(self.filename):
                    raise FileExistsError(self.filename)
        else:
            raise ValueError(f"mode must be 'r', 'w', 'x' or 'w-' (got {mode!r})")

    def _check_writable(self):
        if self.mode == "r":
            raise ValueError("the file is open read-only")
        if self._closed:
            raise ValueError("the file is closed")

    # --- reading ------------------------------------------------------------------
    def _load(self, data):
        rd = _Reader(data)
        seen = {}

        def build(node, addr):
            msgs = rd.messages(addr)
            node._attrs.update(rd.attributes(msgs))
            for name, child_addr in rd.group_links(msgs).items():
                if child_addr in seen:
                    node._links[name] = seen[child_addr]
                    continue
                cm = rd.messages(child_addr)
                kinds = {t for t, _, _ in cm}
                if kinds & {0x11, 0x02, 0x06, 0x0A} and 0x08 not in kinds:
                    g = Group(self, node._child_name(name))
                    seen[child_addr] = g
                    node._links[name] = g
                    build(g, child_addr)
                else:
                    dt_body = next(body for t, _, body in cm if t == 0x03)
                    sp_body = next(body for t, _, body in cm if t == 0x01)
                    dt, _ = _decode_dtype(dt_body, 0)
                    shape = _decode_space(sp_body, 0)
                    raw = rd.read_raw(cm, dt, shape)
                    ds = Dataset(self, node._child_name(name), rd.to_array(raw, dt, shape), dt)
                    if not isinstance(ds._data, np.ndarray):
                        ds._data = np.asarray(ds._data, dtype=object if isinstance(dt, _VlenStr) else None)
                    ds._attrs.update(rd.attributes(cm))
                    seen[child_addr] = ds
                    node._links[name] = ds

        build(self, rd.root_header)

    # --- writing ------------------------------------------------------------------
    def close(self):
        if self._closed:
            return
        if self.mode != "r":
            meta, arrays = _Writer().layout(self)  # laid out first: an error leaves no file behind
            with open(self.filename, "wb") as fh:
                fh.write(meta)
                for arr in arrays:  # streamed from the arrays themselves, no copies
                    fh.write(arr.reshape(-1).view(np.uint8).data)
                    fh.write(b"\x00" * (_pad8(arr.nbytes) - arr.nbytes))
        self._closed = True

    def flush(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __repr__(self):
        return f'<HDF5 file "{self.filename}" (mode {self.mode})>'


# ============================================================================
# writing
# ============================================================================
class _Writer:
    """Lays out a File tree: superblock, then for each group its object header,
    B-tree node, symbol-table nodes and local heap, each dataset's object header
    (variable-length string data beside it), the global heap collections of the
    strings, and last the numeric dataset payloads, written from the arrays
    themselves."""

    def __init__(self):
        self.buf = bytearray()
        self.gcols = []   # [(address, [bytes objects], size)]
        self.vlen_refs = []
        # numeric dataset payloads: (file offset of the layout message's address
        # field, array); placed after all metadata and streamed from the arrays
        self.external = []

    def alloc(self, n):
        addr = len(self.buf)
        self.buf += b"\x00" * _pad8(n)
        return addr

    def put(self, addr, data):
        self.buf[addr:addr + len(data)] = data

    # --- variable-length strings: collected first, written at the end --------
    def vlen_encode(self, values, enc):
        """16-byte heap IDs for each string; the collection addresses are
        patched in when the collections are laid out."""
        out = bytearray()
        for v in values:
            s = v.encode("utf-8") if isinstance(v, str) else bytes(v)
            if not self.gcols or self.gcols[-1][2] + 16 + _pad8(len(s)) > _GCOL_MIN - 32:
                self.gcols.append([None, [], 16])
            col = self.gcols[-1]
            col[1].append(s)
            col[2] += 16 + _pad8(len(s))
            self.vlen_refs.append((len(self.gcols) - 1, len(col[1])))
            out += struct.pack("<IQI", len(s), 0, len(col[1]))
        return bytes(out)

    def _raw(self, data, dt):
        if isinstance(dt, _VlenStr):
            flat = np.asarray(data, dtype=object).ravel()
            return self.vlen_encode(list(flat), dt.encoding), True
        return np.ascontiguousarray(data, dtype=dt).tobytes(), False

    @staticmethod
    def _message(mtype, body, flags=0):
        body = body + b"\x00" * (_pad8(len(body)) - len(body))
        return struct.pack("<HHB3x", mtype, len(body), flags) + body

    def _attr_messages(self, node, patches):
        out = []
        for name, value in node._attrs.items():
            arr, dt = _as_storable(value)
            nm = name.encode("utf-8") + b"\x00"
            tb = _encode_dtype(dt)
            sb = _encode_space(np.shape(arr))
            raw, is_vlen = self._raw(arr, dt)
            head = struct.pack("<BBHHH", 1, 0, len(nm), len(tb), len(sb))
            body = head + nm.ljust(_pad8(len(nm)), b"\x00") + tb.ljust(_pad8(len(tb)), b"\x00") \
                + sb.ljust(_pad8(len(sb)), b"\x00")
            data_off = len(body)
            body += raw
            out.append((0x0C, body, (data_off, len(raw)) if is_vlen else None))
        return out

    def _header(self, msgs):
        """A version-1 object header holding msgs [(type, body, vlen patch)];
        returns (address, {message index: body offset in the file})."""
        encoded = [self._message(t, b, 1 if t in (0x03, 0x05) else 0) for t, b, _ in msgs]
        size = sum(len(e) for e in encoded)
        # libhdf5 gives a header at least room for a few messages; a NIL
        # message fills the tail
        tail = max(0, 24 - size)
        if tail:
            encoded.append(self._message(0x0000, b"\x00" * (tail - 8)))
            size = sum(len(e) for e in encoded)
        addr = self.alloc(16 + size)
        self.put(addr, struct.pack("<BBHII4x", 1, 0, len(encoded), 1, size))
        p = addr + 16
        body_at = []
        for e in encoded:
            self.put(p, e)
            body_at.append(p + 8)
            p += len(e)
        return addr, body_at

    def layout(self, root: File):
        """(metadata bytes, numeric payload arrays): the file is the metadata
        followed by each array padded to 8 bytes, in order."""
        self.alloc(96)  # superblock with the root symbol-table entry
        self.vlen_sites = []  # (file offset of the vlen IDs, count)
        root_addr, btree, heap = self._group(root)
        self._write_gcols()
        addr = len(self.buf)
        for site, arr in self.external:
            struct.pack_into("<Q", self.buf, site, addr)
            addr += _pad8(arr.nbytes)
        eof = addr
        sb = bytearray(_SIG)
        sb += bytes([0, 0, 0, 0, 0, 8, 8, 0])
        sb += struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
        sb += struct.pack("<QQII", 0, root_addr, 1, 0) + struct.pack("<QQ", btree, heap)
        self.put(0, bytes(sb))
        return self.buf, [arr for _, arr in self.external]

    def _group(self, g: Group):
        """Writes the group's subtree; returns (header, B-tree, local heap)."""
        # children first, so that their addresses are known
        entries = []
        for name, child in g._links.items():
            if isinstance(child, Group):
                addr, c_tree, c_heap = self._group(child)
                scratch = (1, struct.pack("<QQ", c_tree, c_heap))
            else:
                addr = self._dataset(child)
                scratch = (0, b"\x00" * 16)
            entries.append((name.encode("utf-8"), addr, scratch))
        entries.sort(key=lambda e: e[0])
        if len(entries) > 2 * _LEAF_K * 2 * _INTERNAL_K:
            raise ValueError(f"a group holds at most {2 * _LEAF_K * 2 * _INTERNAL_K} links here")
        # local heap of names: "" at offset 0, then each name, 8-byte aligned,
        # and a free block at the end (libhdf5 keeps one)
        heap_data = bytearray(8)
        offsets = []
        for name, _, _ in entries:
            offsets.append(len(heap_data))
            heap_data += name + b"\x00"
            heap_data += b"\x00" * (_pad8(len(heap_data)) - len(heap_data))
        free_off = len(heap_data)
        heap_data += struct.pack("<QQ", 1, 16)  # last free block, 16 bytes
        # symbol-table nodes of at most 2K entries each
        nodes = [list(range(i, min(i + 2 * _LEAF_K, len(entries)))) for i in range(0, len(entries), 2 * _LEAF_K)]
        if not nodes:
            nodes = [[]]
        snod_addrs = []
        for idxs in nodes:
            a = self.alloc(_SNOD_SIZE)
            rec = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(idxs)))
            for i in idxs:
                cache, pad = entries[i][2]
                rec += struct.pack("<QQII", offsets[i], entries[i][1], cache, 0) + pad
            self.put(a, bytes(rec))
            snod_addrs.append(a)
        tree = self.alloc(_TREE_SIZE)
        rec = bytearray(b"TREE" + bytes([0, 0]) + struct.pack("<H", len(nodes) if entries else 0))
        rec += struct.pack("<QQ", _UNDEF, _UNDEF)
        if entries:
            rec += struct.pack("<Q", 0)
            for idxs, a in zip(nodes, snod_addrs):
                rec += struct.pack("<QQ", a, offsets[idxs[-1]])
        self.put(tree, bytes(rec))
        heap_seg = self.alloc(len(heap_data))
        self.put(heap_seg, bytes(heap_data))
        heap = self.alloc(32)
        self.put(heap, b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap_data), free_off, heap_seg))
        msgs = [(0x11, struct.pack("<QQ", tree, heap), None)] + self._attr_messages(g, None)
        hdr, body_at = self._header(msgs)
        self._note_vlen_sites(msgs, body_at)
        return hdr, tree, heap

    def _note_vlen_sites(self, msgs, body_at):
        for (t, body, patch), at in zip(msgs, body_at):
            if patch is not None:
                off, length = patch
                self.vlen_sites.append((at + off, length // 16))

    def _dataset(self, ds: Dataset) -> int:
        arr, dt = ds._data, ds.dtype
        shape = np.shape(arr)
        ext = None
        data_addr = _UNDEF
        if isinstance(dt, _VlenStr):
            raw, _ = self._raw(arr, dt)
            nbytes = len(raw)
            if raw:
                data_addr = self.alloc(nbytes)
                self.put(data_addr, raw)
                self.vlen_sites.append((data_addr, nbytes // 16))
        else:
            ext = np.ascontiguousarray(arr, dtype=dt)
            nbytes = ext.nbytes  # its address is set when the metadata is complete
        fill = bytes([2, 2, 2, 1]) + struct.pack("<I", 0)
        layout = bytes([3, 1]) + struct.pack("<QQ", data_addr, nbytes)
        msgs = [(0x01, _encode_space(shape), None), (0x03, _encode_dtype(dt), None), (0x05, fill, None),
                (0x08, layout, None)] + self._attr_messages(ds, None)
        hdr, body_at = self._header(msgs)
        self._note_vlen_sites(msgs, body_at)
        if ext is not None and nbytes:
            self.external.append((body_at[3] + 2, ext))
        return hdr

    def _write_gcols(self):
        addrs = []
        for col in self.gcols:
            objs = col[1]
            size = max(_GCOL_MIN, col[2] + 16)
            a = self.alloc(size)
            rec = bytearray(b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", size))
            for k, s in enumerate(objs, start=1):
                rec += struct.pack("<HHIQ", k, 0, 0, len(s)) + s + b"\x00" * (_pad8(len(s)) - len(s))
            free = size - len(rec)
            rec += struct.pack("<HHIQ", 0, 0, 0, free)
            self.put(a, bytes(rec))
            addrs.append(a)
        # patch the collection addresses into every heap ID, in write order
        refs = iter(self.vlen_refs)
        for site, count in self.vlen_sites:
            for k in range(count):
                col, _idx = next(refs)
                struct.pack_into("<Q", self.buf, site + 16 * k + 4, addrs[col])
