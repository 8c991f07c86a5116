"""HDF5 files without h5py: the subset the result files use.

The reference writes its pruning results, threshold schemes and periodograms
with h5py (``io/cands.py:277-411``, ``detection/thresholding.py``,
``periodogram.py``). h5py and libhdf5 are not available here, so this module
writes and reads HDF5 itself, following the published HDF5 File Format
Specification (version 3.0 of the document; the structures below are its
"version 0" superblock family, readable by every libhdf5 since 1.4):

- superblock version 0 (8-byte offsets and lengths);
- version 1 object headers, with continuation blocks when read;
- groups as symbol tables (a version 1 B-tree of symbol-table nodes over a
  local heap of link names); compact new-style groups (link messages) are
  read as well;
- datasets with contiguous storage (written), contiguous, compact or chunked
  storage with the deflate, shuffle and fletcher32 filters (read);
- datatypes: integers, IEEE floats, fixed-length strings, variable-length
  UTF-8 strings (in a global heap collection), compound types of those;
- attributes (message versions 1 to 3) on groups and datasets.

A file is read whole into a ``Group`` tree and written whole from one, which
suits files of a few MB; ``File`` gives the h5py-style handle the result
writer uses (``attrs``, ``create_group``, ``create_dataset``, ``copy``).
"""

from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"
LEAF_K = 4  # entries per symbol-table node: 2 * LEAF_K
NODE_K = 16  # children per group B-tree node: 2 * NODE_K
GCOL_MIN = 4096  # smallest global heap collection


def _pad8(n: int) -> int:
    return (n + 7) & ~7


# ---------------------------------------------------------------------------
# in-memory tree
# ---------------------------------------------------------------------------


class Dataset:
    """A dataset: a numpy array (object arrays of str for variable-length
    strings) and its attributes."""

    def __init__(self, data, attrs: dict | None = None) -> None:
        self.data = _as_array(data)
        self.attrs: dict = dict(attrs or {})

    def __getitem__(self, key):
        return self.data[key]

    def __array__(self, dtype=None, copy=None):
        return self.data if dtype is None else self.data.astype(dtype)

    def __len__(self) -> int:
        return len(self.data)

    @property
    def shape(self) -> tuple:
        return self.data.shape

    @property
    def dtype(self):
        return self.data.dtype


class Group:
    """A group: named members (groups and datasets) in insertion order, and
    attributes. Paths with '/' reach nested members."""

    def __init__(self) -> None:
        self.members: dict[str, Group | Dataset] = {}
        self.attrs: dict = {}

    def _walk(self, path: str, create: bool = False) -> tuple[Group, str]:
        parts = [p for p in path.split("/") if p]
        if not parts:
            msg = "empty path"
            raise KeyError(msg)
        g = self
        for p in parts[:-1]:
            nxt = g.members.get(p)
            if nxt is None and create:
                nxt = g.members[p] = Group()
            if not isinstance(nxt, Group):
                raise KeyError(path)
            g = nxt
        return g, parts[-1]

    def __getitem__(self, path: str):
        g, name = self._walk(path)
        if name not in g.members:
            raise KeyError(path)
        return g.members[name]

    def __contains__(self, path: str) -> bool:
        try:
            self[path]
        except KeyError:
            return False
        return True

    def __iter__(self):
        return iter(list(self.members))

    def __len__(self) -> int:
        return len(self.members)

    def keys(self):
        return list(self.members)

    def items(self):
        return list(self.members.items())

    def create_group(self, path: str) -> Group:
        g, name = self._walk(path, create=True)
        if name in g.members:
            msg = f"{path!r} already exists"
            raise ValueError(msg)
        g.members[name] = Group()
        return g.members[name]

    def require_group(self, path: str) -> Group:
        if path in self:
            g = self[path]
            if not isinstance(g, Group):
                msg = f"{path!r} is not a group"
                raise TypeError(msg)
            return g
        return self.create_group(path)

    def create_dataset(self, path: str, data=None, **_ignored) -> Dataset:
        """A dataset of ``data``. Storage keywords (``compression``,
        ``chunks``, ...) are accepted and ignored: datasets are written
        contiguous."""
        g, name = self._walk(path, create=True)
        if name in g.members:
            msg = f"{path!r} already exists"
            raise ValueError(msg)
        g.members[name] = Dataset(data)
        return g.members[name]

    def copy(self, source, dest: Group, name: str | None = None) -> None:
        """Deep copy of ``source`` (a path in this group, or a member) into
        group ``dest`` under ``name`` (default: the source's own name)."""
        if isinstance(source, str):
            obj = self[source]
            default = source.rstrip("/").split("/")[-1]
        else:
            obj, default = source, None
        name = name or default
        if not name:
            msg = "copy of an object needs a name"
            raise ValueError(msg)
        if name in dest.members:
            msg = f"{name!r} already exists"
            raise ValueError(msg)
        dest.members[name] = _deep_copy(obj)


def _deep_copy(obj):
    if isinstance(obj, Dataset):
        return Dataset(obj.data.copy(), dict(obj.attrs))
    g = Group()
    g.attrs = dict(obj.attrs)
    for k, v in obj.members.items():
        g.members[k] = _deep_copy(v)
    return g


def _as_array(data) -> np.ndarray:
    """numpy form of a value to store: str and lists of str become object
    arrays (variable-length UTF-8), bytes become fixed-length strings."""
    if isinstance(data, Dataset):
        return data.data
    if isinstance(data, str):
        return np.array(data, dtype=object)
    if isinstance(data, (list, tuple)) and data and all(isinstance(x, str) for x in data):
        return np.array(list(data), dtype=object)
    a = np.asarray(data)
    if a.dtype.kind == "U":
        return a.astype(object)
    return a


class File(Group):
    """An HDF5 file as an in-memory tree: read whole on opening (modes "r",
    "a", "r+"), written whole on closing (modes "w", "w-", "x", "a", "r+")."""

    def __init__(self, path, mode: str = "r") -> None:
        super().__init__()
        self.path = Path(path)
        if mode not in ("r", "r+", "a", "w", "w-", "x"):
            msg = f"invalid mode {mode!r}"
            raise ValueError(msg)
        self.mode = mode
        exists = self.path.exists()
        if mode in ("w-", "x") and exists:
            msg = f"{self.path} already exists"
            raise FileExistsError(msg)
        if mode in ("r", "r+") or (mode == "a" and exists):
            root = read_file(self.path)
            self.members, self.attrs = root.members, root.attrs
        self._open = True

    def close(self) -> None:
        if self._open and self.mode != "r":
            write_file(self.path, self)
        self._open = False

    def __enter__(self) -> File:
        return self

    def __exit__(self, *exc) -> None:
        self.close()


# ---------------------------------------------------------------------------
# datatypes
# ---------------------------------------------------------------------------


def _dt_fixed(size: int, signed: bool) -> bytes:
    return struct.pack("<BBBBIHH", 0x10, 0x08 if signed else 0x00, 0, 0, size, 0, 8 * size)


_FLOAT_LAYOUT = {2: (15, 10, 5, 0, 10, 15), 4: (31, 23, 8, 0, 23, 127),
                 8: (63, 52, 11, 0, 52, 1023)}


def _dt_float(size: int) -> bytes:
    sign, eloc, esize, mloc, msize, bias = _FLOAT_LAYOUT[size]
    return struct.pack("<BBBBIHHBBBBI", 0x11, 0x20, sign, 0, size, 0, 8 * size, eloc, esize,
                       mloc, msize, bias)


def _dt_fixed_string(size: int) -> bytes:
    return struct.pack("<BBBBI", 0x13, 0x00, 0, 0, size)  # null-terminated, ASCII


def _dt_vlen_string() -> bytes:
    # variable-length string (type 1), null-terminated, UTF-8; element:
    # length (4), global heap collection address (8), object index (4)
    return struct.pack("<BBBBI", 0x19, 0x01, 0x01, 0, 16) + _dt_fixed(1, False)


def _dt_bool() -> bytes:
    """numpy bool as h5py stores it: an enumeration over int8 with members
    FALSE = 0 and TRUE = 1 (names padded to 8 bytes in version 1)."""
    return (struct.pack("<BBBBI", 0x18, 2, 0, 0, 1) + _dt_fixed(1, True) +
            b"FALSE\0\0\0" + b"TRUE\0\0\0\0" + bytes([0, 1]))


def _dtype_message(dt: np.dtype) -> bytes:
    """Datatype message (format version 1) of a numpy dtype."""
    if dt.names is not None:
        body = b""
        for name in dt.names:
            sub, off = dt.fields[name][:2]
            if sub.shape:
                msg = "array members of compound types are not supported"
                raise TypeError(msg)
            nm = name.encode("utf-8") + b"\0"
            body += nm + b"\0" * (_pad8(len(nm)) - len(nm))
            body += struct.pack("<IB3xI4x16x", off, 0, 0)
            body += _dtype_message(sub)
        n = len(dt.names)
        return struct.pack("<BBBBI", 0x16, n & 0xFF, n >> 8, 0, dt.itemsize) + body
    if dt.kind == "b":
        return _dt_bool()
    if dt.kind in "iu":
        return _dt_fixed(dt.itemsize, dt.kind == "i")
    if dt.kind == "f" and dt.itemsize in _FLOAT_LAYOUT:
        return _dt_float(dt.itemsize)
    if dt.kind == "S":
        return _dt_fixed_string(max(1, dt.itemsize))
    if dt.kind == "O":
        return _dt_vlen_string()
    msg = f"dtype {dt} is not supported"
    raise TypeError(msg)


class _Reader:
    """Byte access with the file's base address."""

    def __init__(self, buf: bytes) -> None:
        self.buf = buf
        self.base = 0

    def at(self, addr: int, n: int) -> bytes:
        a = self.base + addr
        if addr == UNDEF or a < 0 or a + n > len(self.buf):
            msg = f"address {addr:#x} + {n} outside the file"
            raise ValueError(msg)
        return self.buf[a:a + n]

    def u(self, addr: int, fmt: str):
        return struct.unpack_from("<" + fmt, self.buf, self.base + addr)


def _decode_dtype(b: bytes, p: int) -> tuple[dict, int]:
    """A datatype message at b[p:]: a description dict and the end offset."""
    cv, f0, f1, f2, size = struct.unpack_from("<BBBBI", b, p)
    cls, ver = cv & 0x0F, cv >> 4
    q = p + 8
    flags = f0 | (f1 << 8) | (f2 << 16)
    if cls == 0:  # fixed-point
        q += 4
        order = ">" if flags & 1 else "<"
        return {"np": np.dtype(f"{order}{'i' if flags & 8 else 'u'}{size}")}, q
    if cls == 1:  # floating point
        q += 12
        order = ">" if flags & 1 else "<"
        if size not in (2, 4, 8):
            msg = f"float of {size} bytes"
            raise TypeError(msg)
        return {"np": np.dtype(f"{order}f{size}")}, q
    if cls == 2:  # time: stored as integers
        q += 2
        return {"np": np.dtype(f"<u{size}")}, q
    if cls == 3:  # fixed-length string
        return {"np": np.dtype(f"S{size}"), "str": True}, q
    if cls == 4:  # bitfield
        q += 4
        return {"np": np.dtype(f"<u{size}")}, q
    if cls == 5:  # opaque
        tag_end = b.index(b"\0", q)
        q = q + _pad8(tag_end - q + 1)
        return {"np": np.dtype(f"V{size}")}, q
    if cls == 6:  # compound
        n = flags & 0xFFFF
        names, formats, offsets = [], [], []
        for _ in range(n):
            end = b.index(b"\0", q)
            name = b[q:end].decode("utf-8")
            if ver < 3:
                q += _pad8(end - q + 1)
                off = struct.unpack_from("<I", b, q)[0]
                q += 4
                if ver == 1:
                    q += 28  # dimensionality, permutation, dimension sizes
            else:
                q = end + 1
                nb = 1 if size < 256 else 2 if size < 65536 else 3 if size < 2**24 else 4
                off = int.from_bytes(b[q:q + nb], "little")
                q += nb
            sub, q = _decode_dtype(b, q)
            if "vlen" in sub:
                msg = "variable-length members of compound types are not supported"
                raise TypeError(msg)
            names.append(name)
            formats.append(sub["np"])
            offsets.append(off)
        return {"np": np.dtype({"names": names, "formats": formats, "offsets": offsets,
                                "itemsize": size})}, q
    if cls == 8:  # enumeration: the base integer type (h5py's FALSE/TRUE: bool)
        base, q2 = _decode_dtype(b, q)
        n = flags & 0xFFFF
        names = []
        for _ in range(n):
            end = b.index(b"\0", q2)
            names.append(b[q2:end])
            q2 = end + 1 if ver >= 3 else q2 + _pad8(end - q2 + 1)
        values = np.frombuffer(b[q2:q2 + n * base["np"].itemsize], base["np"])
        q2 += n * base["np"].itemsize
        if base["np"].itemsize == 1 and dict(zip(names, values.tolist())) == {b"FALSE": 0,
                                                                               b"TRUE": 1}:
            return {"np": np.dtype(np.bool_)}, q2
        return {"np": base["np"]}, q2
    if cls == 9:  # variable length
        base, q = _decode_dtype(b, q)
        return {"np": np.dtype(object), "vlen": "str" if (flags & 0x0F) == 1 else "seq",
                "base": base}, q
    if cls == 10:  # array
        nd = b[q]
        q += 1 if ver >= 3 else 4
        dims = struct.unpack_from(f"<{nd}I", b, q)
        q += 4 * nd
        if ver < 3:
            q += 4 * nd  # permutation indices
        base, q = _decode_dtype(b, q)
        return {"np": np.dtype((base["np"], dims))}, q
    msg = f"datatype class {cls} is not supported"
    raise TypeError(msg)


# ---------------------------------------------------------------------------
# writer
# ---------------------------------------------------------------------------


class _Writer:
    def __init__(self) -> None:
        self.out = bytearray(96)  # the superblock, written last
        self.strings: list[bytes] = []  # global heap objects, in index order
        self.gcol_addr = UNDEF
        self.gcol_size = 0

    def alloc(self, data: bytes) -> int:
        addr = len(self.out)
        self.out += data
        self.out += b"\0" * (_pad8(len(self.out)) - len(self.out))
        return addr

    # variable-length strings ---------------------------------------------------
    def collect(self, obj) -> int:
        """Bytes of the global heap objects of every variable-length string
        under obj."""
        n = sum(self._string_bytes(_as_array(v)) for v in obj.attrs.values())
        if isinstance(obj, Dataset):
            return n + self._string_bytes(obj.data)
        return n + sum(self.collect(m) for m in obj.members.values())

    @staticmethod
    def _string_bytes(a: np.ndarray) -> int:
        if a.dtype.kind != "O":
            return 0
        n = 0
        for s in a.reshape(-1):
            if not isinstance(s, str):
                msg = "object arrays hold str only (variable-length strings)"
                raise TypeError(msg)
            b = len(s.encode("utf-8"))
            n += 16 + _pad8(b) if b else 0
        return n

    def reserve_gcol(self, nbytes: int) -> None:
        """One global heap collection for every string, filled as the
        strings are encoded (index order = encoding order)."""
        if nbytes == 0:
            return
        self.gcol_size = max(GCOL_MIN, 16 + nbytes + 16)
        self.gcol_addr = self.alloc(b"\0" * self.gcol_size)

    def fill_gcol(self) -> None:
        if self.gcol_addr == UNDEF:
            return
        body = bytearray(b"GCOL" + bytes([1, 0, 0, 0]) + struct.pack("<Q", self.gcol_size))
        for i, s in enumerate(self.strings, start=1):
            body += struct.pack("<HH4xQ", i, 1, len(s)) + s + b"\0" * (_pad8(len(s)) - len(s))
        free = self.gcol_size - len(body)
        assert free >= 16
        body += struct.pack("<HH4xQ", 0, 0, free)  # the free space object
        self.out[self.gcol_addr:self.gcol_addr + len(body)] = body

    def raw(self, a: np.ndarray) -> bytes:
        """The stored bytes of an array (little-endian; strings through the
        global heap)."""
        if a.dtype.kind == "O":
            out = bytearray()
            for s in a.reshape(-1):
                b = s.encode("utf-8")
                if not b:  # an empty string has no heap object
                    out += struct.pack("<IQI", 0, 0, 0)
                    continue
                self.strings.append(b)
                out += struct.pack("<IQI", len(b), self.gcol_addr, len(self.strings))
            return bytes(out)
        if a.dtype.names is None and a.dtype.byteorder == ">":
            a = a.astype(a.dtype.newbyteorder("<"))
        return np.ascontiguousarray(a).tobytes()

    # messages ------------------------------------------------------------------
    @staticmethod
    def msg(mtype: int, data: bytes, flags: int = 0) -> bytes:
        data = data + b"\0" * (_pad8(len(data)) - len(data))
        return struct.pack("<HHB3x", mtype, len(data), flags) + data

    @staticmethod
    def dataspace(shape: tuple) -> bytes:
        return struct.pack("<BBB5x", 1, len(shape), 0) + b"".join(
            struct.pack("<Q", d) for d in shape)

    def attribute(self, name: str, value) -> bytes:
        a = _as_array(value)
        nm = name.encode("utf-8") + b"\0"
        dt = _dtype_message(a.dtype)
        ds = self.dataspace(a.shape)
        body = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds))
        for part in (nm, dt, ds):
            body += part + b"\0" * (_pad8(len(part)) - len(part))
        body += self.raw(a)
        return self.msg(0x0C, body)

    def header(self, messages: list[bytes]) -> int:
        body = b"".join(messages)
        return self.alloc(struct.pack("<BBHII4x", 1, 0, len(messages), 1, len(body)) + body)

    # objects -------------------------------------------------------------------
    def dataset(self, d: Dataset) -> int:
        a = d.data
        raw = self.raw(a)
        addr = self.alloc(raw) if raw else UNDEF
        msgs = [self.msg(0x01, self.dataspace(a.shape)),
                self.msg(0x03, _dtype_message(a.dtype), flags=1),
                self.msg(0x05, bytes([2, 2, 2, 0]), flags=1),  # fill value: none defined
                self.msg(0x08, struct.pack("<BBQQ", 3, 1, addr, len(raw)))]
        msgs += [self.attribute(k, v) for k, v in d.attrs.items()]
        return self.header(msgs)

    def group(self, g: Group) -> tuple[int, int, int]:
        """Writes a group's members, its name heap, symbol-table nodes and
        B-tree, then its object header; returns (header, B-tree, heap)."""
        children = {name: (self.group(m)[0] if isinstance(m, Group) else self.dataset(m))
                    for name, m in g.members.items()}
        names = sorted(children, key=lambda s: s.encode("utf-8"))
        heap = bytearray(8)  # offset 0: the empty name
        offs = {}
        for n in names:
            offs[n] = len(heap)
            bn = n.encode("utf-8") + b"\0"
            heap += bn + b"\0" * (_pad8(len(bn)) - len(bn))
        data_addr = self.alloc(bytes(heap))
        heap_addr = self.alloc(b"HEAP" + bytes([0, 0, 0, 0]) +
                               struct.pack("<QQQ", len(heap), 1, data_addr))
        # symbol-table nodes, full
        per = 2 * LEAF_K
        nodes = []  # (address, left key, right key)
        for i in range(0, len(names), per):
            chunk = names[i:i + per]
            body = b"SNOD" + struct.pack("<BBH", 1, 0, len(chunk))
            for n in chunk:
                body += struct.pack("<QQI4x16x", offs[n], children[n], 0)
            body += b"\0" * (40 * (per - len(chunk)))
            nodes.append((self.alloc(body), offs[chunk[-1]]))
        btree = self.btree(nodes)
        hdr = self.header([self.msg(0x11, struct.pack("<QQ", btree, heap_addr))] +
                          [self.attribute(k, v) for k, v in g.attrs.items()])
        return hdr, btree, heap_addr

    def btree(self, children: list[tuple[int, int]]) -> int:
        """Group B-tree (version 1, type 0) over (child address, right key)
        pairs, left key of the first child 0 (the empty name); returns the
        root address."""
        level = 0
        per = 2 * NODE_K
        node_size = 24 + per * 8 + (per + 1) * 8
        if not children:
            return self.alloc(b"TREE" + struct.pack("<BBHQQ", 0, 0, 0, UNDEF, UNDEF) +
                              b"\0" * (node_size - 24))
        while True:
            groups = [children[i:i + per] for i in range(0, len(children), per)]
            start = len(self.out)
            addrs = [start + k * node_size for k in range(len(groups))]
            upper = []
            left_key = 0
            for k, grp in enumerate(groups):
                body = b"TREE" + struct.pack(
                    "<BBHQQ", 0, level, len(grp), addrs[k - 1] if k else UNDEF,
                    addrs[k + 1] if k + 1 < len(groups) else UNDEF)
                body += struct.pack("<Q", left_key)
                for child, right in grp:
                    body += struct.pack("<QQ", child, right)
                body += b"\0" * (node_size - len(body))
                got = self.alloc(body)
                assert got == addrs[k]
                upper.append((got, grp[-1][1]))
                left_key = grp[-1][1]
            if len(upper) == 1:
                return upper[0][0]
            children = upper
            level += 1

    def finish(self, root_hdr: int, btree: int, heap: int) -> bytes:
        eof = len(self.out)
        sb = SIGNATURE + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack(
            "<HHI", LEAF_K, NODE_K, 0)
        sb += struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
        sb += struct.pack("<QQI4xQQ", 0, root_hdr, 1, btree, heap)  # root symbol-table entry
        assert len(sb) == 96
        self.out[:96] = sb
        return bytes(self.out)


def write_file(path, root: Group) -> None:
    """Write the tree under ``root`` (its attributes included) as an HDF5 file."""
    w = _Writer()
    w.reserve_gcol(w.collect(root))
    hdr, btree, heap = w.group(root)
    w.fill_gcol()
    data = w.finish(hdr, btree, heap)
    tmp = Path(str(path) + ".tmp")
    tmp.write_bytes(data)
    tmp.replace(path)


# ---------------------------------------------------------------------------
# reader
# ---------------------------------------------------------------------------


class _FileReader(_Reader):
    def __init__(self, buf: bytes) -> None:
        super().__init__(buf)
        off = 0
        while True:  # the superblock is at 0, 512, 1024, ...
            if off + 8 > len(buf):
                msg = "not an HDF5 file (no signature)"
                raise ValueError(msg)
            if buf[off:off + 8] == SIGNATURE:
                break
            off = 512 if off == 0 else off * 2
        ver = buf[off + 8]
        if ver not in (0, 1):
            msg = f"superblock version {ver} is not supported (0 and 1 are)"
            raise ValueError(msg)
        so, sl = buf[off + 13], buf[off + 14]
        if (so, sl) != (8, 8):
            msg = f"offsets of {so} and lengths of {sl} bytes are not supported"
            raise ValueError(msg)
        p = off + 24 + (4 if ver == 1 else 0)
        base = struct.unpack_from("<Q", buf, p)[0]
        self.base = base if base != UNDEF else off
        root_entry = p + 32
        self.root_addr = struct.unpack_from("<Q", buf, root_entry + 8)[0]
        self.gcols: dict[int, dict[int, bytes]] = {}

    # global heap -------------------------------------------------------------
    def gheap(self, addr: int, index: int) -> bytes:
        col = self.gcols.get(addr)
        if col is None:
            if self.at(addr, 4) != b"GCOL":
                msg = f"no global heap collection at {addr:#x}"
                raise ValueError(msg)
            size = self.u(addr + 8, "Q")[0]
            data = self.at(addr, size)
            col = {}
            q = 16
            while q + 16 <= size:
                idx, _, osize = struct.unpack_from("<HH4xQ", data, q)
                if idx == 0:
                    break
                col[idx] = data[q + 16:q + 16 + osize]
                q += 16 + _pad8(osize)
            self.gcols[addr] = col
        return col[index]

    # arrays --------------------------------------------------------------------
    def array(self, raw: bytes, dt: dict, shape: tuple) -> np.ndarray:
        n = int(np.prod(shape, dtype=np.int64)) if shape else 1
        if "vlen" in dt:
            out = np.empty(n, dtype=object)
            for i in range(n):
                length, caddr, idx = struct.unpack_from("<IQI", raw, 16 * i)
                if caddr in (0, UNDEF) or length == 0 and idx == 0:
                    obj = b""
                else:
                    obj = self.gheap(caddr, idx)
                if dt["vlen"] == "str":
                    out[i] = obj[:length].decode("utf-8")
                else:
                    base = dt["base"]["np"]
                    out[i] = np.frombuffer(obj[:length * base.itemsize], base).copy()
            return out.reshape(shape)
        a = np.frombuffer(raw[:n * dt["np"].itemsize], dtype=dt["np"]).copy()
        if a.dtype.names is None and a.dtype.byteorder == ">":
            a = a.astype(a.dtype.newbyteorder("<"))
        return a.reshape(shape)

    # object headers ------------------------------------------------------------
    def messages(self, addr: int) -> list[tuple[int, bytes]]:
        """(type, data) of every message of the object header at addr,
        continuation blocks followed."""
        out: list[tuple[int, bytes]] = []
        if self.at(addr, 4) == b"OHDR":
            return self._messages_v2(addr, out)
        ver, _, nmsg, _, size = self.u(addr, "BBHII")
        if ver != 1:
            msg = f"object header version {ver} at {addr:#x}"
            raise ValueError(msg)
        blocks = [(addr + 16, size)]
        seen = set()
        while blocks and len(out) < nmsg:
            start, length = blocks.pop(0)
            if start in seen:
                msg = f"object header at {addr:#x}: continuation blocks form a cycle"
                raise ValueError(msg)
            seen.add(start)
            data = self.at(start, length)
            q = 0
            while q + 8 <= length and len(out) < nmsg:
                mtype, msize, _ = struct.unpack_from("<HHB", data, q)
                body = data[q + 8:q + 8 + msize]
                q += 8 + msize
                if mtype == 0x10:
                    blocks.append(struct.unpack_from("<QQ", body))
                out.append((mtype, body))
        return out

    def _messages_v2(self, addr: int, out: list) -> list:
        flags = self.at(addr + 5, 1)[0]
        q = addr + 6
        if flags & 0x20:
            q += 16  # access, modification, change, birth times
        if flags & 0x10:
            q += 4  # attribute phase change values
        nsz = 1 << (flags & 3)
        size = int.from_bytes(self.at(q, nsz), "little")
        q += nsz
        blocks = [(q, size)]
        track = bool(flags & 0x04)
        seen = set()
        while blocks:
            start, length = blocks.pop(0)
            if start in seen:
                msg = f"object header at {addr:#x}: continuation blocks form a cycle"
                raise ValueError(msg)
            seen.add(start)
            data = self.at(start, length)
            p = 0
            while p + 4 <= length:
                mtype, msize, _ = struct.unpack_from("<BHB", data, p)
                p += 4 + (2 if track else 0)
                body = data[p:p + msize]
                p += msize
                if mtype == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", body)
                    blocks.append((caddr + 4, clen - 8))  # "OCHK" ... checksum
                out.append((mtype, body))
        return out

    def attribute(self, body: bytes) -> tuple[str, np.ndarray]:
        ver = body[0]
        flags = body[1]
        nlen, tlen, slen = struct.unpack_from("<HHH", body, 2)
        q = 8
        if ver == 3:
            q += 1  # name character set
        name = body[q:q + nlen].split(b"\0")[0].decode("utf-8")
        q += _pad8(nlen) if ver == 1 else nlen
        if flags & 1:
            msg = f"attribute {name!r}: shared datatypes are not supported"
            raise TypeError(msg)
        dt, _ = _decode_dtype(body, q)
        q += _pad8(tlen) if ver == 1 else tlen
        shape = self.dataspace(body[q:q + slen])
        q += _pad8(slen) if ver == 1 else slen
        return name, self.array(body[q:], dt, shape)

    @staticmethod
    def dataspace(body: bytes) -> tuple:
        ver, nd, flags = body[0], body[1], body[2]
        if ver == 1:
            q = 8
        else:
            if body[3] == 2:  # null dataspace
                return (0,)
            q = 4
        return tuple(struct.unpack_from(f"<{nd}Q", body, q)) if nd else ()

    # objects -------------------------------------------------------------------
    def obj(self, addr: int, seen: set | None = None):
        seen = set() if seen is None else seen
        if addr in seen:
            msg = f"object at {addr:#x} is linked twice (hard-link cycles are not supported)"
            raise ValueError(msg)
        seen = seen | {addr}
        msgs = self.messages(addr)
        kinds = {t for t, _ in msgs}
        attrs = {}
        for t, b in msgs:
            if t == 0x0C:
                k, v = self.attribute(b)
                attrs[k] = v[()] if v.ndim == 0 and v.dtype.kind == "O" else v
            elif t == 0x15 and struct.unpack_from("<Q", b, 2 + (2 if b[1] & 1 else 0))[0] \
                    != UNDEF:
                msg = "dense attribute storage is not supported"
                raise NotImplementedError(msg)
        if 0x11 in kinds or 0x02 in kinds or 0x06 in kinds:
            g = Group()
            g.attrs = attrs
            for name, child in self.links(msgs):
                g.members[name] = self.obj(child, seen)
            return g
        if 0x08 not in kinds:
            msg = f"object at {addr:#x} is neither a group nor a dataset"
            raise ValueError(msg)
        body = dict(msgs)
        shape = self.dataspace(body[0x01])
        dt, _ = _decode_dtype(body[0x03], 0)
        raw = self.layout(body[0x08], shape, dt, body.get(0x0B))
        return Dataset(self.array(raw, dt, shape), attrs)

    def links(self, msgs) -> list[tuple[str, int]]:
        out = []
        for t, b in msgs:
            if t == 0x11:
                btree, heap = struct.unpack_from("<QQ", b)
                out += self.symbol_table(btree, heap)
            elif t == 0x02:
                flags = b[1]
                q = 2 + (8 if flags & 1 else 0)
                fheap = struct.unpack_from("<Q", b, q)[0]
                if fheap != UNDEF:
                    msg = "dense link storage is not supported"
                    raise NotImplementedError(msg)
            elif t == 0x06:
                link = self.link(b)
                if link is not None:
                    out.append(link)
        return out

    @staticmethod
    def link(b: bytes):
        flags = b[1]
        q = 2
        ltype = 0
        if flags & 0x08:
            ltype = b[q]
            q += 1
        if flags & 0x04:
            q += 8  # creation order
        if flags & 0x10:
            q += 1  # name character set
        nsz = 1 << (flags & 3)
        nlen = int.from_bytes(b[q:q + nsz], "little")
        q += nsz
        name = b[q:q + nlen].decode("utf-8")
        q += nlen
        if ltype != 0:
            return None  # soft and external links are skipped
        return name, struct.unpack_from("<Q", b, q)[0]

    def symbol_table(self, btree: int, heap: int) -> list[tuple[str, int]]:
        if self.at(heap, 4) != b"HEAP":
            msg = f"no local heap at {heap:#x}"
            raise ValueError(msg)
        dsize, _, daddr = self.u(heap + 8, "QQQ")
        names = self.at(daddr, dsize)
        out = []
        seen: set[int] = set()

        def walk(node: int) -> None:
            if node in seen:
                msg = f"group B-tree node {node:#x} is reached twice"
                raise ValueError(msg)
            seen.add(node)
            if self.at(node, 4) != b"TREE":
                msg = f"no B-tree node at {node:#x}"
                raise ValueError(msg)
            ntype, level, used = self.u(node + 4, "BBH")
            if ntype != 0:
                msg = "group B-tree of the wrong type"
                raise ValueError(msg)
            for i in range(used):
                child = self.u(node + 24 + 8 + 16 * i, "Q")[0]
                if level > 0:
                    walk(child)
                    continue
                if self.at(child, 4) != b"SNOD":
                    msg = f"no symbol-table node at {child:#x}"
                    raise ValueError(msg)
                nsym = self.u(child + 6, "H")[0]
                for k in range(nsym):
                    noff, ohdr = self.u(child + 8 + 40 * k, "QQ")
                    out.append((names[noff:names.index(b"\0", noff)].decode("utf-8"), ohdr))

        walk(btree)
        return out

    def layout(self, b: bytes, shape: tuple, dt: dict, pipeline: bytes | None) -> bytes:
        ver = b[0]
        esize = 16 if "vlen" in dt else dt["np"].itemsize
        nbytes = int(np.prod(shape, dtype=np.int64)) * esize if shape else esize
        if ver in (1, 2):
            nd, cls = b[1], b[2]
            q = 8
            addr = struct.unpack_from("<Q", b, q)[0] if cls != 0 else UNDEF
            q += 8 if cls != 0 else 0
            dims = struct.unpack_from(f"<{nd}I", b, q)
            q += 4 * nd
            if cls == 0:
                n = struct.unpack_from("<I", b, q)[0]
                return b[q + 4:q + 4 + n]
            if cls == 1:
                return self.at(addr, nbytes) if addr != UNDEF else b"\0" * nbytes
            return self.chunked(addr, dims, shape, esize, pipeline)
        if ver != 3:
            msg = f"layout message version {ver} is not supported"
            raise ValueError(msg)
        cls = b[1]
        if cls == 0:
            n = struct.unpack_from("<H", b, 2)[0]
            return b[4:4 + n]
        if cls == 1:
            addr, size = struct.unpack_from("<QQ", b, 2)
            return self.at(addr, nbytes) if addr != UNDEF else b"\0" * nbytes
        if cls == 2:
            nd = b[2]
            addr = struct.unpack_from("<Q", b, 3)[0]
            dims = struct.unpack_from(f"<{nd}I", b, 11)
            return self.chunked(addr, dims, shape, esize, pipeline)
        msg = f"layout class {cls} is not supported"
        raise ValueError(msg)

    def filters(self, pipeline: bytes | None) -> list[tuple[int, tuple]]:
        if pipeline is None:
            return []
        ver, n = pipeline[0], pipeline[1]
        q = 8 if ver == 1 else 2
        out = []
        for _ in range(n):
            fid = struct.unpack_from("<H", pipeline, q)[0]
            q += 2
            nlen = 0
            if ver == 1 or fid >= 256:
                nlen = struct.unpack_from("<H", pipeline, q)[0]
                q += 2
            _, nval = struct.unpack_from("<HH", pipeline, q)
            q += 4
            q += _pad8(nlen) if ver == 1 else nlen
            vals = struct.unpack_from(f"<{nval}I", pipeline, q)
            q += 4 * nval + (4 if ver == 1 and nval % 2 else 0)
            out.append((fid, vals))
        return out

    def chunked(self, btree: int, dims: tuple, shape: tuple, esize: int,
                pipeline: bytes | None) -> bytes:
        cshape = tuple(dims[:-1])
        nd = len(cshape)
        out = np.zeros(shape if shape else (1,), dtype=f"V{esize}")
        flist = self.filters(pipeline)
        csize = int(np.prod(cshape, dtype=np.int64)) * esize
        if btree == UNDEF:
            return out.tobytes()
        key_size = 8 + 8 * (nd + 1)
        seen: set[int] = set()

        def unfilter(data: bytes, mask: int) -> bytes:
            for k in range(len(flist) - 1, -1, -1):
                if mask & (1 << k):
                    continue
                fid, vals = flist[k]
                if fid == 1:
                    data = zlib.decompress(data)
                elif fid == 2:
                    size = vals[0] if vals else esize
                    arr = np.frombuffer(data, np.uint8)
                    n = len(arr) // size
                    body = arr[:n * size].reshape(size, n).T.reshape(-1)
                    data = body.tobytes() + arr[n * size:].tobytes()
                elif fid == 3:
                    data = data[:-4]
                else:
                    msg = f"filter {fid} is not supported"
                    raise NotImplementedError(msg)
            return data

        def walk(node: int) -> None:
            if node in seen:
                msg = f"chunk B-tree node {node:#x} is reached twice"
                raise ValueError(msg)
            seen.add(node)
            if self.at(node, 4) != b"TREE":
                msg = f"no B-tree node at {node:#x}"
                raise ValueError(msg)
            ntype, level, used = self.u(node + 4, "BBH")
            if ntype != 1:
                msg = "chunk B-tree of the wrong type"
                raise ValueError(msg)
            q = node + 24
            for _ in range(used):
                nbytes, mask = self.u(q, "II")
                offs = self.u(q + 8, f"{nd}Q")
                child = self.u(q + key_size, "Q")[0]
                q += key_size + 8
                if level > 0:
                    walk(child)
                    continue
                data = unfilter(self.at(child, nbytes), mask)[:csize]
                chunk = np.frombuffer(data, dtype=f"V{esize}").reshape(cshape)
                sl = tuple(slice(o, min(o + c, s)) for o, c, s in zip(offs, cshape, shape))
                src = tuple(slice(0, s.stop - s.start) for s in sl)
                out[sl] = chunk[src]

        walk(btree)
        return out.tobytes()


def read_file(path) -> Group:
    """The tree of an HDF5 file (superblock version 0 or 1)."""
    r = _FileReader(Path(path).read_bytes())
    root = r.obj(r.root_addr)
    if not isinstance(root, Group):
        msg = "the root object is not a group"
        raise ValueError(msg)
    return root


__all__ = ["Dataset", "File", "Group", "read_file", "write_file"]
