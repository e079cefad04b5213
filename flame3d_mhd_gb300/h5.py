"""HDF5 files of the reference (metrics.h5, mesh.h5, plot, checkpoint and average files)
without an HDF5 library: a reader and a writer of the classic ("earliest") HDF5 format that
HDF5.jl writes by default, restated from the published HDF5 file-format specification.

Reader: version-0/1 superblock (with or without a user block), symbol-table groups (version-1
B-tree of type 0, symbol-table nodes, local heap), version-1 object headers with continuation
blocks, dataspace v1/v2, fixed-point / floating-point / string datatypes, data layout v1-v3
(compact, contiguous, chunked through a version-1 B-tree of type 1) and the deflate, shuffle
and Fletcher-32 filters; attributes (message 0x000C, v1) of those types. Files written with
the newer format (superblock v2/v3, "OHDR" object headers) raise ValueError.

Writer: a version-0 superblock at offset 0, the root group as a symbol table, datasets
contiguous or chunked (optionally shuffled and deflated; at most 64 chunks, one leaf of the
chunk B-tree), scalars as rank-0 dataspaces (HDF5.jl's `file["NG"] = NG`).

Arrays are C order. HDF5.jl stores a Julia array of size (n1, ..., nk) with file dimensions
(nk, ..., n1), so the file's dimensions are those of this package's arrays: a Julia
(Nx, Ny, Nz) array is (Nz, Ny, Nx) here and in the file.
"""
from __future__ import annotations

import mmap
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIG = b"\x89HDF\r\n\x1a\n"
HEAP_FREE_NULL = 1  # end of a local heap's free list on disk
GROUP_LEAF_K, GROUP_INTERNAL_K, ISTORE_K = 4, 16, 32  # library defaults (the v0 superblock has no istore K)

# message types
M_NIL, M_DATASPACE, M_DATATYPE, M_FILL_OLD, M_FILL, M_LAYOUT, M_FILTERS, M_ATTRIBUTE = 0, 1, 3, 4, 5, 8, 11, 12
M_CONTINUATION, M_SYMBOL_TABLE, M_MTIME = 0x10, 0x11, 0x12
F_DEFLATE, F_SHUFFLE, F_FLETCHER32 = 1, 2, 3


def _u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def _pad8(n):
    return (n + 7) & ~7


# ----------------------------------------------------------------------------------- reader


class Dataset:
    """One dataset: `shape`, `dtype`, `attrs`, `layout`, `filters` and `read()` (a numpy array
    that owns its data)."""

    def __init__(self, f: "H5File", name: str, msgs: list):
        self.f, self.name = f, name
        self.shape, self.dtype, self.layout, self.filters = None, None, None, []
        self.attrs = {}
        for mtype, body in msgs:
            if mtype == M_DATASPACE:
                self.shape = _dataspace(body, f.L)
            elif mtype == M_DATATYPE:
                self.dtype = _datatype(body)[0]
            elif mtype == M_LAYOUT:
                self.layout = _layout(body, f.O, f.L)
            elif mtype == M_FILTERS:
                self.filters = _filters(body)
            elif mtype == M_ATTRIBUTE:
                k, v = _attribute(body, f)
                self.attrs[k] = v
        if self.shape is None or self.dtype is None or self.layout is None:
            raise ValueError(f"{name}: not a dataset (dataspace, datatype or layout missing)")

    def read(self) -> np.ndarray:
        kind = self.layout[0]
        n = int(np.prod(self.shape, dtype=np.int64))
        if kind == "compact":
            return np.frombuffer(self.layout[1], self.dtype, n).reshape(self.shape).copy()
        if kind == "contiguous":
            addr = self.layout[1]
            if addr == UNDEF:
                return np.zeros(self.shape, self.dtype)
            a = self.f.abs(addr)
            return np.frombuffer(self.f.buf, self.dtype, n, a).reshape(self.shape).copy()
        return self._read_chunked()

    def _read_chunked(self) -> np.ndarray:
        _, btree, cdims = self.layout
        rank = len(self.shape)
        cshape, esize = tuple(cdims[:rank]), cdims[rank]
        if esize != self.dtype.itemsize:
            raise ValueError(f"{self.name}: chunk element size {esize} != {self.dtype.itemsize}")
        out = np.zeros(self.shape, self.dtype)
        if btree == UNDEF:
            return out
        for size, mask, offs, addr in self.f.chunk_entries(btree, rank + 1):
            raw = bytes(self.f.buf[self.f.abs(addr):self.f.abs(addr) + size])
            for i in reversed(range(len(self.filters))):
                fid, cd = self.filters[i]
                if mask >> i & 1:
                    continue
                raw = _unfilter(fid, cd, raw, esize)
            c = np.frombuffer(raw, self.dtype, int(np.prod(cshape))).reshape(cshape)
            sl = tuple(slice(o, min(o + s, d)) for o, s, d in zip(offs, cshape, self.shape))
            out[sl] = c[tuple(slice(0, s.stop - s.start) for s in sl)]
        return out


class H5File:
    """A read-only view of a classic-format HDF5 file: `keys()`, `[name]` -> numpy array,
    `dataset(name)` -> Dataset (attributes, layout), `group(path)` -> dict of entries."""

    def __init__(self, path: str):
        self._fh = open(path, "rb")
        try:
            self.buf = mmap.mmap(self._fh.fileno(), 0, access=mmap.ACCESS_READ)
        except ValueError:  # an empty file
            self._fh.close()
            raise ValueError(f"{path}: empty file")
        b = self.buf
        sb = next((o for o in [0] + [512 << i for i in range(20)] if o + 8 <= len(b) and b[o:o + 8] == SIG), None)
        if sb is None:
            self.close()
            raise ValueError(f"{path}: no HDF5 signature")
        ver = b[sb + 8]
        if ver not in (0, 1):
            self.close()
            raise ValueError(f"{path}: superblock version {ver} (only the classic v0/v1 format is read)")
        self.O, self.L = b[sb + 13], b[sb + 14]
        if self.O != 8 or self.L != 8:
            self.close()
            raise ValueError(f"{path}: offsets of {self.O} and lengths of {self.L} bytes (8 and 8 are read)")
        p = sb + 24 + (4 if ver == 1 else 0)  # v1 adds the indexed-storage K and 2 reserved bytes
        self.base = _u(b, p, 8)
        self.eof = _u(b, p + 16, 8)
        self.root = self._entry(p + 32)

    def close(self):
        try:
            self.buf.close()
        finally:
            self._fh.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def abs(self, addr: int) -> int:
        return self.base + addr

    # -- structures
    def _entry(self, p):
        """A symbol-table entry: (name offset, object header address, cache type, scratch)."""
        b = self.buf
        return _u(b, p, 8), _u(b, p + 8, 8), _u(b, p + 16, 4), bytes(b[p + 24:p + 40])

    def messages(self, addr: int) -> list:
        """The (type, body) messages of the version-1 object header at `addr`."""
        b, p = self.buf, self.abs(addr)
        if b[p] != 1:
            raise ValueError(f"object header version {b[p]} at {addr} (only version 1 is read)")
        nmsg, size = _u(b, p + 2, 2), _u(b, p + 8, 4)
        blocks, out = [(p + 16, size)], []
        while blocks and len(out) < nmsg:
            q, n = blocks.pop(0)
            end = q + n
            while q + 8 <= end and len(out) < nmsg:
                mtype, msize = _u(b, q, 2), _u(b, q + 2, 2)
                body = bytes(b[q + 8:q + 8 + msize])
                q += 8 + msize
                if mtype == M_CONTINUATION:
                    blocks.append((self.abs(_u(body, 0, 8)), _u(body, 8, 8)))
                out.append((mtype, body))
        return [(t, m) for t, m in out if t not in (M_NIL, M_CONTINUATION)]

    def _heap(self, addr):
        b, p = self.buf, self.abs(addr)
        if b[p:p + 4] != b"HEAP":
            raise ValueError(f"no local heap at {addr}")
        return self.abs(_u(b, p + 24, 8))

    def _name(self, heap_data, off):
        b = self.buf
        e = b.find(b"\0", heap_data + off)
        return bytes(b[heap_data + off:e]).decode("utf-8")

    def _btree_children(self, addr, ntype, key_size):
        """(key before, child, key after) of every leaf-level child of the v1 B-tree at `addr`."""
        b, p = self.buf, self.abs(addr)
        if b[p:p + 4] != b"TREE" or b[p + 4] != ntype:
            raise ValueError(f"no B-tree node of type {ntype} at {addr}")
        level, used = b[p + 5], _u(b, p + 6, 2)
        q = p + 24
        for _ in range(used):
            key, child = q, _u(b, q + key_size, 8)
            q += key_size + 8
            if level == 0:
                yield key, child, q
            else:
                yield from self._btree_children(child, ntype, key_size)

    def group(self, addr: int | None = None) -> dict:
        """{name: object header address} of the symbol-table group at `addr` (the root by default)."""
        msgs = self.messages(self.root[1] if addr is None else addr)
        st = next((m for t, m in msgs if t == M_SYMBOL_TABLE), None)
        if st is None:
            raise ValueError("not a symbol-table group (new-style link messages are not read)")
        btree, heap = _u(st, 0, 8), _u(st, 8, 8)
        hd = self._heap(heap)
        out = {}
        for _, snod, _ in self._btree_children(btree, 0, self.L):
            p = self.abs(snod)
            if self.buf[p:p + 4] != b"SNOD":
                raise ValueError(f"no symbol-table node at {snod}")
            for i in range(_u(self.buf, p + 6, 2)):
                noff, oh, _, _ = self._entry(p + 8 + 40 * i)
                out[self._name(hd, noff)] = oh
        return out

    def chunk_entries(self, btree: int, ndims: int):
        """(stored size, filter mask, chunk offsets, address) of every chunk under `btree`."""
        ks = 8 + 8 * ndims
        for key, child, _ in self._btree_children(btree, 1, ks):
            b = self.buf
            offs = tuple(_u(b, key + 8 + 8 * d, 8) for d in range(ndims - 1))
            yield _u(b, key, 4), _u(b, key + 4, 4), offs, child

    def _resolve(self, path: str) -> int:
        addr = self.root[1]
        for part in [s for s in path.split("/") if s]:
            g = self.group(addr)
            if part not in g:
                raise KeyError(path)
            addr = g[part]
        return addr

    def keys(self) -> list:
        return list(self.group().keys())

    def dataset(self, path: str) -> Dataset:
        return Dataset(self, path, self.messages(self._resolve(path)))

    def __getitem__(self, path: str) -> np.ndarray:
        return self.dataset(path).read()

    def __contains__(self, path: str) -> bool:
        try:
            self._resolve(path)
            return True
        except KeyError:
            return False


def _dataspace(m, L):
    ver, rank, flags = m[0], m[1], m[2]
    if ver == 1:
        p = 8
    elif ver == 2:
        if m[3] == 2:  # null dataspace
            return None
        p = 4
    else:
        raise ValueError(f"dataspace version {ver}")
    return tuple(_u(m, p + L * i, L) for i in range(rank))


def _datatype(m):
    """(numpy dtype, byte size) of a datatype message body."""
    cls, ver = m[0] & 0x0F, m[0] >> 4
    bits, size = m[1] | m[2] << 8 | m[3] << 16, _u(m, 4, 4)
    order = ">" if bits & 1 else "<"
    if cls == 0:
        return np.dtype(f"{order}{'i' if bits & 8 else 'u'}{size}"), size
    if cls == 1:
        if bits & 0x40:
            raise ValueError("VAX floating point")
        return np.dtype(f"{order}f{size}"), size
    if cls == 3:
        return np.dtype(f"S{size}"), size
    raise ValueError(f"datatype class {cls} (version {ver}) is not read")


def _layout(m, O, L):
    ver = m[0]
    if ver in (1, 2):
        rank, cls = m[1], m[2]
        p = 8
        addr = None
        if cls != 0:
            addr = _u(m, p, O)
            p += O
        dims = [_u(m, p + 4 * i, 4) for i in range(rank)]
        p += 4 * rank
        if cls == 0:
            n = _u(m, p, 4)
            return ("compact", m[p + 4:p + 4 + n])
        if cls == 1:
            return ("contiguous", addr)
        return ("chunked", addr, dims)
    if ver == 3:
        cls = m[1]
        if cls == 0:
            n = _u(m, 2, 2)
            return ("compact", m[4:4 + n])
        if cls == 1:
            return ("contiguous", _u(m, 2, O))
        if cls == 2:
            nd = m[2]
            return ("chunked", _u(m, 3, O), [_u(m, 3 + O + 4 * i, 4) for i in range(nd)])
    raise ValueError(f"data layout version {ver} is not read")


def _filters(m):
    ver, n = m[0], m[1]
    out, p = [], (8 if ver == 1 else 2)
    for _ in range(n):
        fid = _u(m, p, 2)
        if ver == 1 or fid >= 256:
            nlen = _u(m, p + 2, 2)
            p += 2
        else:
            nlen = 0
        nval = _u(m, p + 4, 2)
        p += 6
        p += _pad8(nlen) if ver == 1 else nlen
        cd = [_u(m, p + 4 * i, 4) for i in range(nval)]
        p += 4 * nval
        if ver == 1 and nval % 2:
            p += 4
        out.append((fid, cd))
    return out


def _unfilter(fid, cd, raw, esize):
    if fid == F_DEFLATE:
        return zlib.decompress(raw)
    if fid == F_SHUFFLE:
        e = cd[0] if cd else esize
        n = len(raw) // e
        body = np.frombuffer(raw[:n * e], np.uint8).reshape(e, n).T.tobytes()
        return body + raw[n * e:]
    if fid == F_FLETCHER32:
        return raw[:-4]
    raise ValueError(f"filter {fid} is not supported")


def _attribute(m, f):
    ver = m[0]
    if ver != 1:
        raise ValueError(f"attribute version {ver} is not read")
    nlen, tlen, slen = _u(m, 2, 2), _u(m, 4, 2), _u(m, 6, 2)
    p = 8
    name = m[p:p + nlen].split(b"\0")[0].decode("utf-8")
    p += _pad8(nlen)
    dt, size = _datatype(m[p:p + tlen])
    p += _pad8(tlen)
    shape = _dataspace(m[p:p + slen], f.L) or ()
    p += _pad8(slen)
    n = int(np.prod(shape, dtype=np.int64)) if shape else 1
    v = np.frombuffer(m[p:p + n * size], dt, n)
    if dt.kind == "S":
        return name, v[0].split(b"\0")[0].decode("utf-8") if n == 1 else [s.decode("utf-8") for s in v]
    return name, v.reshape(shape) if shape else v[0]


def read(path: str) -> dict:
    """{name: numpy array} of every dataset in the root group of `path` (copied out)."""
    with H5File(path) as f:
        return {k: f[k] for k in f.keys()}


# ----------------------------------------------------------------------------------- writer


def _dtype_msg(dt: np.dtype) -> bytes:
    dt = np.dtype(dt)
    if dt.byteorder == ">":
        raise ValueError("big-endian arrays are not written")
    if dt.kind == "f" and dt.itemsize in (4, 8):
        sign, exp_loc, exp_size, mant, bias = ((31, 23, 8, 23, 127) if dt.itemsize == 4 else (63, 52, 11, 52, 1023))
        return (bytes([0x11, 0x20, sign, 0]) + struct.pack("<I", dt.itemsize)
                + struct.pack("<HHBBBBI", 0, 8 * dt.itemsize, exp_loc, exp_size, 0, mant, bias))
    if dt.kind in "iu" and dt.itemsize in (1, 2, 4, 8):
        return (bytes([0x10, 0x08 if dt.kind == "i" else 0, 0, 0]) + struct.pack("<I", dt.itemsize)
                + struct.pack("<HH", 0, 8 * dt.itemsize))
    raise ValueError(f"dtype {dt} is not written (float32/64 and integers are)")


def _dataspace_msg(shape) -> bytes:
    return bytes([1, len(shape), 0, 0]) + b"\0" * 4 + b"".join(struct.pack("<Q", d) for d in shape)


def _message(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = body + b"\0" * (_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(msgs: list[bytes]) -> bytes:
    data = b"".join(msgs)
    return struct.pack("<BxHII4x", 1, len(msgs), 1, len(data)) + data


def _shuffle(raw: bytes, e: int) -> bytes:
    n = len(raw) // e
    return np.frombuffer(raw[:n * e], np.uint8).reshape(n, e).T.tobytes() + raw[n * e:]


class _Alloc:
    """Sequential space: blocks appended after the superblock, each at an 8-byte boundary."""

    def __init__(self, start):
        self.end, self.blocks = start, []

    def take(self, n, align=8):
        a = (self.end + align - 1) // align * align
        self.end = a + n
        return a

    def put(self, addr, data):
        self.blocks.append((addr, data))


def write(path: str, datasets: dict, chunks: dict | None = None, deflate: int | None = None,
          shuffle: bool = False) -> str:
    """Write {name: array} as root-group datasets of a new classic-format HDF5 file.

    Arrays keep their C-order shape as the file's dimensions; 0-d arrays and Python scalars
    become scalar dataspaces. `chunks` maps names to chunk shapes (chunked layout, at most 64
    chunks a dataset); `deflate` (0-9) and `shuffle` apply to the chunked datasets. Names are
    UTF-8 and sorted in the group's B-tree by their bytes, as the library keeps them.
    """
    chunks = chunks or {}
    items = sorted(((k.encode("utf-8"), np.asarray(v).copy(order="C")) for k, v in datasets.items()),
                   key=lambda kv: kv[0])  # a C-order copy that keeps 0-d arrays 0-d
    if len({k for k, _ in items}) != len(items):
        raise ValueError("duplicate names")
    if any(b"/" in k or not k for k, _ in items):
        raise ValueError("names must be non-empty and contain no '/'")
    al = _Alloc(96)

    # local heap of names: "" at 0, then each name NUL-terminated on an 8-byte grid, then a free block
    heap_data, name_off = bytearray(8), {}
    for k, _ in items:
        name_off[k] = len(heap_data)
        heap_data += k + b"\0" * (_pad8(len(k) + 1) - len(k))
    free_off = len(heap_data)
    heap_data += struct.pack("<QQ", HEAP_FREE_NULL, 16)  # one free block of 16 bytes (next: none)
    heap_hdr, heap_seg = al.take(32), al.take(len(heap_data))
    al.put(heap_hdr, b"HEAP" + b"\0" * 4 + struct.pack("<QQQ", len(heap_data), free_off, heap_seg))
    al.put(heap_seg, bytes(heap_data))

    # datasets: object header then data
    entries = []
    for k, a in items:
        chunked = k.decode("utf-8") in chunks and a.size > 0  # an empty array stays contiguous
        # fill value v2: allocation late (contiguous) or incremental (chunked), written if set,
        # the default value (defined, size 0), as the library writes it
        fill = bytes([2, 3 if chunked else 2, 2, 1]) + struct.pack("<I", 0)
        msgs = [_message(M_DATASPACE, _dataspace_msg(a.shape)), _message(M_DATATYPE, _dtype_msg(a.dtype), 1),
                _message(M_FILL, fill, 1)]
        raw = a.tobytes()
        if chunked:
            cshape = tuple(int(c) for c in chunks[k.decode("utf-8")])
            if len(cshape) != a.ndim or a.ndim == 0 or any(c < 1 or c > d for c, d in zip(cshape, a.shape)):
                raise ValueError(f"{k!r}: chunk shape {cshape} for an array of shape {a.shape}")
            grid = [range(0, d, c) for d, c in zip(a.shape, cshape)]
            origins = np.stack(np.meshgrid(*grid, indexing="ij"), -1).reshape(-1, a.ndim)
            if len(origins) > 2 * ISTORE_K:
                raise ValueError(f"{k!r}: {len(origins)} chunks (at most {2 * ISTORE_K} are written)")
            pipe = []
            if shuffle and a.itemsize > 1:
                pipe.append((F_SHUFFLE, [a.itemsize]))
            if deflate is not None:
                pipe.append((F_DEFLATE, [int(deflate)]))
            if pipe:
                fm = bytes([1, len(pipe)]) + b"\0" * 6
                for fid, cd in pipe:
                    fm += struct.pack("<HHHH", fid, 0, 1, len(cd))  # both filters optional
                    fm += b"".join(struct.pack("<I", c) for c in cd) + (b"\0" * 4 if len(cd) % 2 else b"")
                msgs.append(_message(M_FILTERS, fm))
            nd = a.ndim + 1
            ks = 8 + 8 * nd
            node_size = 24 + (2 * ISTORE_K + 1) * ks + 2 * ISTORE_K * 8
            btree = al.take(node_size)
            node = bytearray(b"TREE" + bytes([1, 0]) + struct.pack("<HQQ", len(origins), UNDEF, UNDEF))
            for o in origins:
                sl = tuple(slice(int(s), int(s) + c) for s, c in zip(o, cshape))
                c = np.zeros(cshape, a.dtype)
                part = a[sl]
                c[tuple(slice(0, n) for n in part.shape)] = part
                data = c.tobytes()
                for fid, cd in pipe:
                    data = _shuffle(data, cd[0]) if fid == F_SHUFFLE else zlib.compress(data, cd[0])
                addr = al.take(len(data))
                al.put(addr, data)
                node += struct.pack("<II", len(data), 0) + b"".join(struct.pack("<Q", int(v)) for v in o)
                node += struct.pack("<Q", 0) + struct.pack("<Q", addr)
            # the final key: the last chunk's offset plus the chunk dimensions
            node += struct.pack("<II", 0, 0) + b"".join(struct.pack("<Q", int(o) + c)
                                                         for o, c in zip(origins[-1], cshape)) + struct.pack("<Q", 0)
            node += b"\0" * (node_size - len(node))
            al.put(btree, bytes(node))
            lay = bytes([3, 2, nd]) + struct.pack("<Q", btree) + b"".join(struct.pack("<I", c) for c in cshape)
            lay += struct.pack("<I", a.itemsize)
        else:
            addr = al.take(len(raw)) if raw else UNDEF
            if raw:
                al.put(addr, raw)
            lay = bytes([3, 1]) + struct.pack("<QQ", addr, len(raw))
        msgs.append(_message(M_LAYOUT, lay))
        oh = _object_header(msgs)
        oh_addr = al.take(len(oh))
        al.put(oh_addr, oh)
        entries.append((k, oh_addr))

    # symbol-table nodes of up to 2K entries, indexed by one leaf of the group B-tree
    cap = 2 * GROUP_LEAF_K
    snods = [entries[i:i + cap] for i in range(0, len(entries), cap)] or [[]]
    if len(snods) > 2 * GROUP_INTERNAL_K:
        raise ValueError(f"{len(entries)} datasets (at most {2 * GROUP_INTERNAL_K * cap} are written)")
    snod_size = 8 + cap * 40
    node_size = 24 + (2 * GROUP_INTERNAL_K + 1) * 8 + 2 * GROUP_INTERNAL_K * 8
    btree = al.take(node_size)
    node = bytearray(b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(snods) if entries else 0, UNDEF, UNDEF))
    node += struct.pack("<Q", 0)  # key 0: the empty name
    for s in snods if entries else []:
        sa = al.take(snod_size)
        body = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(s)))
        for k, oh in s:
            body += struct.pack("<QQI4x", name_off[k], oh, 0) + b"\0" * 16
        body += b"\0" * (snod_size - len(body))
        al.put(sa, bytes(body))
        node += struct.pack("<Q", sa) + struct.pack("<Q", name_off[s[-1][0]])
    node += b"\0" * (node_size - len(node))
    al.put(btree, bytes(node))

    root = _object_header([_message(M_SYMBOL_TABLE, struct.pack("<QQ", btree, heap_hdr))])
    root_addr = al.take(len(root))
    al.put(root_addr, root)
    eof = al.end
    sb = (SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", GROUP_LEAF_K, GROUP_INTERNAL_K, 0)
          + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF)
          + struct.pack("<QQI4x", 0, root_addr, 1) + struct.pack("<QQ", btree, heap_hdr))
    assert len(sb) == 96
    with open(path, "wb") as f:
        f.write(sb)
        pos = 96
        for addr, data in sorted(al.blocks, key=lambda x: x[0]):
            if addr > pos:
                f.write(b"\0" * (addr - pos))
            f.write(data)
            pos = addr + len(data)
        if eof > pos:
            f.write(b"\0" * (eof - pos))
    return path
