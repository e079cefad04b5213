"""HDF5 files of the reference (metrics.h5, mesh.h5, plot, checkpoint and average files)
without an HDF5 library: a reader and a writer restated from the published HDF5 file-format
specification.

Reader: superblocks v0-v3 (with or without a user block); version-1 object headers and
version-2 ("OHDR"/"OCHK") object headers; groups as symbol tables (v1 B-tree of type 0,
symbol-table nodes, local heap) or as link messages, held in the object header (compact) or
in a fractal heap indexed by a v2 B-tree of link-name hashes (dense; a root direct block or
a root indirect block of direct blocks, a name index of depth 0 or 1); dataspace v1/v2,
fixed-point / floating-point / string datatypes; data layout v1-v4 (compact, contiguous,
chunked through a v1 B-tree, the single-chunk and implicit indexes of v4) and the deflate,
shuffle and Fletcher-32 filters; attributes v1-v3 of those types. Checksums (Jenkins'
lookup3, as the format uses it) are verified on the structures that carry one, except
fractal-heap direct blocks. HDF5.jl creates its links with UTF-8 names, which makes the
library store groups as link messages; both group forms are read.

Writer: by default the classic ("earliest") format every HDF5 library reads: a version-0
superblock at offset 0, the root group as a symbol table, datasets contiguous or chunked
(optionally shuffled and deflated; at most 64 chunks, one leaf of the chunk B-tree), scalars
as rank-0 dataspaces (HDF5.jl's `file["NG"] = NG`). `links=True` stores the root group as
link messages (dense beyond eight links) and `new_format=True` writes a version-2 superblock
and version-2 object headers, with the single-chunk and implicit chunk indexes.

Arrays are C order. HDF5.jl stores a Julia array of size (n1, ..., nk) with file dimensions
(nk, ..., n1), so the file's dimensions are those of this package's arrays: a Julia
(Nx, Ny, Nz) array is (Nz, Ny, Nx) here and in the file.
"""
from __future__ import annotations

import mmap
import os
import struct
import zlib

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIG = b"\x89HDF\r\n\x1a\n"
HEAP_FREE_NULL = 1  # end of a local heap's free list on disk
GROUP_LEAF_K, GROUP_INTERNAL_K, ISTORE_K = 4, 16, 32  # library defaults (the v0 superblock has no istore K)
MAX_COMPACT_LINKS = 8  # the library's default: a ninth link moves a group's links to dense storage

# message types
M_NIL, M_DATASPACE, M_LINK_INFO, M_DATATYPE, M_FILL_OLD, M_FILL, M_LINK = 0, 1, 2, 3, 4, 5, 6
M_LAYOUT, M_GROUP_INFO, M_FILTERS, M_ATTRIBUTE = 8, 10, 11, 12
M_CONTINUATION, M_SYMBOL_TABLE, M_MTIME = 0x10, 0x11, 0x12
F_DEFLATE, F_SHUFFLE, F_FLETCHER32 = 1, 2, 3
BT2_LINK_NAME = 5  # v2 B-tree record type: link-name hash and heap ID


def _u(b, off, n):
    return int.from_bytes(b[off:off + n], "little")


def _pad8(n):
    return (n + 7) & ~7


def _parallel_map(fn, items: list) -> list:
    """fn over items on a thread pool (zlib and numpy copies release the GIL), in order."""
    if len(items) < 2:
        return [fn(x) for x in items]
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=min(len(items), os.cpu_count() or 1)) as ex:
        return list(ex.map(fn, items))


def _rot(x, k):
    return ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF


def lookup3(data: bytes, initval: int = 0) -> int:
    """Bob Jenkins' lookup3 hash (hashlittle, byte-wise), the checksum of HDF5's metadata
    blocks and the hash of its dense link names. The mix and final steps cycle through
    (a, b, c) with the published rotation counts."""
    M = 0xFFFFFFFF
    n = len(data)
    v = [(0xDEADBEEF + n + initval) & M] * 3
    p = 0
    while n > 12:
        for i in range(3):
            v[i] = (v[i] + _u(data, p + 4 * i, 4)) & M
        for i, r in enumerate((4, 6, 8, 16, 19, 4)):  # mix: x -= z; x ^= rot(z, r); z += y
            x, y, z = i % 3, (i + 1) % 3, (i + 2) % 3
            v[x] = ((v[x] - v[z]) & M) ^ _rot(v[z], r)
            v[z] = (v[z] + v[y]) & M
        p += 12
        n -= 12
    if n == 0:
        return v[2]
    tail = bytes(data[p:p + n]) + b"\0" * (12 - n)
    for i in range(3):
        v[i] = (v[i] + _u(tail, 4 * i, 4)) & M
    for i, r in enumerate((14, 11, 25, 16, 4, 14, 24)):  # final: x ^= z; x -= rot(z, r)
        x = (2 + i) % 3
        z = (x + 2) % 3
        v[x] = ((v[x] ^ v[z]) - _rot(v[z], r)) & M
    return v[2]


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
                kv = _attribute(body, f)
                if kv is not None:
                    self.attrs[kv[0]] = kv[1]
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
        rank = len(self.shape)
        cdims = self.layout[2]
        cshape, esize = tuple(cdims[:rank]), cdims[rank]
        if esize != self.dtype.itemsize:
            raise ValueError(f"{self.name}: chunk element size {esize} != {self.dtype.itemsize}")
        out = np.zeros(self.shape, self.dtype)
        if self.layout[1] == UNDEF:
            return out
        if kind == "chunked":
            chunks = self.f.chunk_entries(self.layout[1], rank + 1)
        elif kind == "single":
            size = self.layout[3] if self.layout[3] is not None else int(np.prod(cshape)) * esize
            chunks = [(size, self.layout[4] or 0, (0,) * rank, self.layout[1])]
        else:  # implicit: every chunk at full size, in row-major order of the chunk grid
            cbytes = int(np.prod(cshape)) * esize
            grid = [range(0, d, c) for d, c in zip(self.shape, cshape)]
            origins = np.stack(np.meshgrid(*grid, indexing="ij"), -1).reshape(-1, rank)
            chunks = [(cbytes, 0, tuple(int(v) for v in o), self.layout[1] + i * cbytes)
                      for i, o in enumerate(origins)]
        def place(entry):
            size, mask, offs, addr = entry
            raw = bytes(self.f.buf[self.f.abs(addr):self.f.abs(addr) + size])
            for i in reversed(range(len(self.filters))):
                fid, cd = self.filters[i]
                if mask >> i & 1:
                    continue
                raw = _unfilter(fid, cd, raw, esize)
            c = np.frombuffer(raw, self.dtype, int(np.prod(cshape))).reshape(cshape)
            sl = tuple(slice(o, min(o + s, d)) for o, s, d in zip(offs, cshape, self.shape))
            out[sl] = c[tuple(slice(0, s.stop - s.start) for s in sl)]  # disjoint regions

        _parallel_map(place, list(chunks))
        return out


class H5File:
    """A read-only view of an HDF5 file: `keys()`, `[name]` -> numpy array, `dataset(name)` ->
    Dataset (attributes, layout), `group(addr)` -> {name: object header address}."""

    def __init__(self, path: str):
        self._fh = open(path, "rb")
        try:
            self.buf = mmap.mmap(self._fh.fileno(), 0, access=mmap.ACCESS_READ)
        except ValueError:  # an empty file
            self._fh.close()
            raise ValueError(f"{path}: empty file")
        try:
            self._superblock(path)
        except Exception:
            self.close()
            raise

    def _superblock(self, path):
        b = self.buf
        sb = next((o for o in [0] + [512 << i for i in range(20)] if o + 8 <= len(b) and b[o:o + 8] == SIG), None)
        if sb is None:
            raise ValueError(f"{path}: no HDF5 signature")
        ver = b[sb + 8]
        if ver in (0, 1):
            self.O, self.L = b[sb + 13], b[sb + 14]
        elif ver in (2, 3):
            self.O, self.L = b[sb + 9], b[sb + 10]
        else:
            raise ValueError(f"{path}: superblock version {ver}")
        if self.O != 8 or self.L != 8:
            raise ValueError(f"{path}: offsets of {self.O} and lengths of {self.L} bytes (8 and 8 are read)")
        if ver in (0, 1):
            p = sb + 24 + (4 if ver == 1 else 0)  # v1 adds the indexed-storage K and 2 reserved bytes
            self.base = _u(b, p, 8)
            self.eof = _u(b, p + 16, 8)
            self.root = self._entry(p + 32)
        else:
            p = sb + 12
            self._verify(sb, p + 32, "superblock")
            self.base, self.eof = _u(b, p, 8), _u(b, p + 16, 8)
            self.root = (0, _u(b, p + 24, 8), 0, b"")
        self.version = ver

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

    def _verify(self, start: int, end: int, what: str):
        """The lookup3 checksum stored at `end` covers the bytes [start, end)."""
        if lookup3(self.buf[start:end]) != _u(self.buf, end, 4):
            raise ValueError(f"checksum mismatch in the {what} at {start}")

    # -- object headers
    def _entry(self, p):
        """A symbol-table entry: (name offset, object header address, cache type, scratch)."""
        b = self.buf
        return _u(b, p, 8), _u(b, p + 8, 8), _u(b, p + 16, 4), bytes(b[p + 24:p + 40])

    def messages(self, addr: int) -> list:
        """The (type, body) messages of the object header at `addr` (version 1 or 2)."""
        b, p = self.buf, self.abs(addr)
        if b[p:p + 4] == b"OHDR":
            return self._messages_v2(p)
        if b[p] != 1:
            raise ValueError(f"object header version {b[p]} at {addr}")
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

    def _messages_v2(self, p):
        b = self.buf
        if b[p + 4] != 2:
            raise ValueError(f"OHDR version {b[p + 4]}")
        flags = b[p + 5]
        q = p + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
        csize = 1 << (flags & 3)
        size0 = _u(b, q, csize)
        q += csize
        self._verify(p, q + size0, "object header")
        hsz = 4 + (2 if flags & 0x04 else 0)  # type, size, flags [, creation order]
        blocks, out = [(q, q + size0)], []
        while blocks:
            q, end = blocks.pop(0)
            while q + hsz <= end:
                mtype, msize = b[q], _u(b, q + 1, 2)
                body = bytes(b[q + hsz:q + hsz + msize])
                q += hsz + msize
                if mtype == M_CONTINUATION:
                    c, n = self.abs(_u(body, 0, 8)), _u(body, 8, 8)
                    if b[c:c + 4] != b"OCHK":
                        raise ValueError(f"no OCHK continuation block at {c}")
                    self._verify(c, c + n - 4, "object header continuation")
                    blocks.append((c + 4, c + n - 4))
                out.append((mtype, body))
        return [(t, m) for t, m in out if t not in (M_NIL, M_CONTINUATION)]

    # -- symbol-table groups
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

    def _symbol_table(self, st) -> dict:
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

    # -- dense link storage: fractal heap + v2 B-tree name index
    def _fheap(self, addr) -> dict:
        b, p = self.buf, self.abs(addr)
        if b[p:p + 5] != b"FRHP\0":
            raise ValueError(f"no fractal heap header at {addr}")
        h = {"id_len": _u(b, p + 5, 2), "filter_len": _u(b, p + 7, 2), "max_man": _u(b, p + 10, 4),
             "width": _u(b, p + 110, 2), "start": _u(b, p + 112, 8), "max_direct": _u(b, p + 120, 8),
             "max_bits": _u(b, p + 128, 2), "root": _u(b, p + 132, 8), "rows": _u(b, p + 140, 2)}
        end = p + 142 + ((8 + 4 + h["filter_len"]) if h["filter_len"] else 0)
        self._verify(p, end, "fractal heap header")
        h["off_size"] = (h["max_bits"] + 7) // 8
        h["len_size"] = min((h["max_direct"].bit_length() - 1 + 7) // 8, (h["max_man"].bit_length() - 1) // 8 + 1)
        return h

    def _fheap_object(self, h: dict, hid: bytes) -> bytes:
        if (hid[0] >> 4) & 3:
            raise ValueError("huge and tiny fractal-heap objects are not read")
        off = _u(hid, 1, h["off_size"])
        n = _u(hid, 1 + h["off_size"], h["len_size"])
        if h["rows"] == 0:
            blk, blk_off = h["root"], 0
        else:
            blk, blk_off = self._fheap_block(h, off)
        b, p = self.buf, self.abs(blk)
        if b[p:p + 4] != b"FHDB":
            raise ValueError(f"no fractal heap direct block at {blk}")
        return bytes(b[p + off - blk_off:p + off - blk_off + n])

    def _fheap_block(self, h: dict, off: int) -> tuple[int, int]:
        """(address, heap offset) of the direct block holding heap offset `off`, a child of
        the root indirect block (rows of `width` blocks: start, start, 2 start, 4 start ...)."""
        b, p = self.buf, self.abs(h["root"])
        if b[p:p + 4] != b"FHIB":
            raise ValueError(f"no fractal heap indirect block at {h['root']}")
        q = p + 5 + 8 + h["off_size"]
        W, S = h["width"], h["start"]
        max_drows = (h["max_direct"] // S).bit_length() - 1 + 2
        entry = 8 + ((8 + 4) if h["filter_len"] else 0)
        row_off = 0
        for r in range(min(h["rows"], max_drows)):
            size = S if r == 0 else S << (r - 1)
            for c in range(W):
                start = row_off + c * size
                if start <= off < start + size:
                    addr = _u(b, q + (r * W + c) * entry, 8)
                    if addr == UNDEF:
                        raise ValueError(f"heap offset {off} in an unallocated block")
                    return addr, start
            row_off += W * size
        raise ValueError(f"heap offset {off} lies in a child indirect block (not read)")

    def _bt2_records(self, addr, depth, nrec, node_size, rsize) -> list:
        b, p = self.buf, self.abs(addr)
        if depth == 0:
            if b[p:p + 4] != b"BTLF":
                raise ValueError(f"no v2 B-tree leaf at {addr}")
            end = p + 6 + nrec * rsize
            self._verify(p, end, "v2 B-tree leaf")
            return [bytes(b[p + 6 + i * rsize:p + 6 + (i + 1) * rsize]) for i in range(nrec)]
        if depth > 1:
            raise ValueError("v2 B-trees deeper than one level are not read")
        if b[p:p + 4] != b"BTIN":
            raise ValueError(f"no v2 B-tree internal node at {addr}")
        out = [bytes(b[p + 6 + i * rsize:p + 6 + (i + 1) * rsize]) for i in range(nrec)]
        q = p + 6 + nrec * rsize
        nsz = (((node_size - 10) // rsize).bit_length() + 7) // 8  # bytes of a leaf's record count
        for _ in range(nrec + 1):
            child, cn = _u(b, q, 8), _u(b, q + 8, nsz)
            q += 8 + nsz
            out += self._bt2_records(child, 0, cn, node_size, rsize)
        self._verify(p, q, "v2 B-tree internal node")
        return out

    def _dense_links(self, heap_addr, btree_addr) -> dict:
        h = self._fheap(heap_addr)
        b, p = self.buf, self.abs(btree_addr)
        if b[p:p + 5] != b"BTHD\0" or b[p + 5] != BT2_LINK_NAME:
            raise ValueError(f"no link-name v2 B-tree at {btree_addr}")
        node_size, rsize, depth = _u(b, p + 6, 4), _u(b, p + 10, 2), _u(b, p + 12, 2)
        root, nroot = _u(b, p + 16, 8), _u(b, p + 24, 2)
        self._verify(p, p + 34, "v2 B-tree header")
        out = {}
        if root == UNDEF:
            return out
        for rec in self._bt2_records(root, depth, nroot, node_size, rsize):
            name, target = _link(self._fheap_object(h, rec[4:4 + h["id_len"]]))
            if target is not None:
                out[name] = target
        return out

    def group(self, addr: int | None = None) -> dict:
        """{name: object header address} of the hard links of the group at `addr` (the root
        by default), stored as a symbol table or as link messages (compact or dense)."""
        msgs = self.messages(self.root[1] if addr is None else addr)
        st = next((m for t, m in msgs if t == M_SYMBOL_TABLE), None)
        if st is not None:
            return self._symbol_table(st)
        li = next((m for t, m in msgs if t == M_LINK_INFO), None)
        if li is None:
            raise ValueError("not a group (no symbol-table or link-info message)")
        p = 2 + (8 if li[1] & 1 else 0)
        heap, names = _u(li, p, 8), _u(li, p + 8, 8)
        if heap != UNDEF:
            return self._dense_links(heap, names)
        out = {}
        for t, m in msgs:
            if t == M_LINK:
                name, target = _link(m)
                if target is not None:
                    out[name] = target
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


def _link(m) -> tuple[str, int | None]:
    """(name, object header address) of a link message; the address is None for soft and
    external links."""
    flags = m[1]
    p = 2
    ltype = 0
    if flags & 0x08:
        ltype = m[p]
        p += 1
    if flags & 0x04:
        p += 8  # creation order
    if flags & 0x10:
        p += 1  # character set
    nsz = 1 << (flags & 3)
    nlen = _u(m, p, nsz)
    p += nsz
    name = bytes(m[p:p + nlen]).decode("utf-8")
    p += nlen
    return name, (_u(m, p, 8) if ltype == 0 else None)


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
    if ver in (3, 4):
        cls = m[1]
        if cls == 0:
            n = _u(m, 2, 2)
            return ("compact", m[4:4 + n])
        if cls == 1:
            return ("contiguous", _u(m, 2, O))
        if cls == 2 and ver == 3:
            nd = m[2]
            return ("chunked", _u(m, 3, O), [_u(m, 3 + O + 4 * i, 4) for i in range(nd)])
        if cls == 2:
            flags, nd, enc = m[2], m[3], m[4]
            p = 5
            dims = [_u(m, p + enc * i, enc) for i in range(nd)]
            p += enc * nd
            itype = m[p]
            p += 1
            if itype == 1:  # single chunk
                fsize = fmask = None
                if flags & 2:
                    fsize, fmask = _u(m, p, L), _u(m, p + L, 4)
                    p += L + 4
                return ("single", _u(m, p, O), dims, fsize, fmask)
            if itype == 2:  # implicit
                return ("implicit", _u(m, p, O), dims)
            raise ValueError(f"chunk index type {itype} (fixed / extensible array, v2 B-tree) is not read")
    raise ValueError(f"data layout version {ver} class {m[1]} is not read")


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
    """(name, value) of an attribute message; None for attributes of other types or with a
    shared datatype / dataspace."""
    ver = m[0]
    if ver not in (1, 2, 3) or (ver > 1 and m[1] & 3):
        return None
    nlen, tlen, slen = _u(m, 2, 2), _u(m, 4, 2), _u(m, 6, 2)
    p = 8 + (1 if ver == 3 else 0)
    pad = _pad8 if ver == 1 else (lambda n: n)
    name = bytes(m[p:p + nlen]).split(b"\0")[0].decode("utf-8")
    p += pad(nlen)
    try:
        dt, size = _datatype(m[p:p + tlen])
    except ValueError:
        return None
    p += pad(tlen)
    shape = _dataspace(m[p:p + slen], f.L) or ()
    p += pad(slen)
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


def _link_msg(name: bytes, addr: int) -> bytes:
    """A hard link with a UTF-8 name, as HDF5.jl creates them: version 1, the character set
    present (flag bit 4), the name length in 1, 2 or 4 bytes (flag bits 0-1)."""
    n = len(name)
    code = 0 if n < 1 << 8 else (1 if n < 1 << 16 else 2)
    return bytes([1, 0x10 | code, 1]) + n.to_bytes(1 << code, "little") + name + struct.pack("<Q", addr)


def _message(mtype: int, body: bytes, flags: int = 0) -> bytes:
    """A message of a version-1 object header (8-byte header, body padded to 8 bytes)."""
    body = body + b"\0" * (_pad8(len(body)) - len(body))
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _object_header(msgs: list, v2: bool = False) -> bytes:
    """An object header of (type, body, flags) messages: version 1, or version 2 ("OHDR",
    chunk-0 size in 4 bytes, 4-byte message headers, lookup3 checksum)."""
    if v2:
        body = b"".join(struct.pack("<BHB", t, len(d), fl) + d for t, d, fl in msgs)
        data = b"OHDR" + bytes([2, 0x02]) + struct.pack("<I", len(body)) + body
        return data + struct.pack("<I", lookup3(data))
    enc = [_message(t, d, fl) for t, d, fl in msgs]
    data = b"".join(enc)
    return struct.pack("<BxHII4x", 1, len(enc), 1, len(data)) + data


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


def _dense_links(al: _Alloc, entries: list) -> tuple[int, int]:
    """Dense link storage for [(name, object header address)]: the link messages as objects
    of a fractal heap with one root direct block (checksummed) and their name hashes in a v2
    B-tree of one leaf. Returns (heap header address, B-tree header address)."""
    objs = [_link_msg(k, a) for k, a in entries]
    off_size, len_size, id_len = 4, 2, 7  # heap offsets of 32 bits, objects below 64 KiB
    dhead = 4 + 1 + 8 + off_size + 4  # FHDB, version, heap header, block offset, checksum
    need = dhead + sum(len(o) for o in objs)
    S = 512
    while S < need:
        S *= 2
    if S > 65536:
        raise ValueError("the names do not fit one 64 KiB heap block")
    heap_hdr, dblock = al.take(146), al.take(S)
    block = bytearray(S)
    block[0:5] = b"FHDB\0"
    block[5:13] = struct.pack("<Q", heap_hdr)  # block offset 0 and checksum 0 follow
    ids, p = [], dhead
    for o in objs:
        block[p:p + len(o)] = o
        ids.append(bytes([0]) + p.to_bytes(off_size, "little") + len(o).to_bytes(len_size, "little"))
        p += len(o)
    block[dhead - 4:dhead] = struct.pack("<I", lookup3(bytes(block)))  # over the block, checksum zeroed
    al.put(dblock, bytes(block))
    hdr = (b"FRHP\0" + struct.pack("<HHB", id_len, 0, 0x02) + struct.pack("<I", 4096)
           + struct.pack("<QQQQQQQQQQQQ", 0, UNDEF, S - need, UNDEF, S, S, S, len(objs), 0, 0, 0, 0)
           + struct.pack("<HQQHHQH", 4, S, 65536, 32, 1, dblock, 0))
    al.put(heap_hdr, hdr + struct.pack("<I", lookup3(hdr)))
    # the name index: (hash, heap ID) records ordered by hash, then name
    recs = sorted((lookup3(k), k, hid) for (k, _), hid in zip(entries, ids))
    node_size, rsize = 512, 4 + id_len
    if len(recs) > (node_size - 10) // rsize:
        raise ValueError(f"{len(recs)} links (at most {(node_size - 10) // rsize} are written densely)")
    bt_hdr, leaf = al.take(38), al.take(node_size)
    lf = b"BTLF\0" + bytes([BT2_LINK_NAME]) + b"".join(struct.pack("<I", h) + hid for h, _, hid in recs)
    lf += struct.pack("<I", lookup3(lf))
    al.put(leaf, lf + b"\0" * (node_size - len(lf)))
    bh = (b"BTHD\0" + bytes([BT2_LINK_NAME]) + struct.pack("<IHHBB", node_size, rsize, 0, 100, 40)
          + struct.pack("<QHQ", leaf, len(recs), len(recs)))
    al.put(bt_hdr, bh + struct.pack("<I", lookup3(bh)))
    return heap_hdr, bt_hdr


def write(path: str, datasets: dict, chunks: dict | None = None, deflate: int | None = None,
          shuffle: bool = False, links: bool = False, new_format: bool = False) -> str:
    """Write {name: array} as root-group datasets of a new HDF5 file.

    Arrays keep their C-order shape as the file's dimensions; 0-d arrays and Python scalars
    become scalar dataspaces. `chunks` maps names to chunk shapes (chunked layout, at most 64
    chunks a dataset); `deflate` (0-9) and `shuffle` apply to the chunked datasets. Names are
    UTF-8. The root group is a symbol table (names sorted by their bytes, as the library
    keeps them) or, with `links`, link messages (compact up to eight, dense beyond).
    `new_format`: a version-2 superblock and version-2 object headers; a dataset of one chunk
    then uses the single-chunk index and an unfiltered dataset of several the implicit one.
    """
    chunks = chunks or {}
    items = sorted(((k.encode("utf-8"), np.asarray(v).copy(order="C")) for k, v in datasets.items()),
                   key=lambda kv: kv[0])  # a C-order copy that keeps 0-d arrays 0-d
    if len({k for k, _ in items}) != len(items):
        raise ValueError("duplicate names")
    if any(b"/" in k or not k for k, _ in items):
        raise ValueError("names must be non-empty and contain no '/'")
    al = _Alloc(96)

    # datasets: object header then data
    entries = []
    for k, a in items:
        chunked = k.decode("utf-8") in chunks and a.size > 0  # an empty array stays contiguous
        # fill value v2: allocation late (contiguous) or incremental (chunked), written if set,
        # the default value (defined, size 0), as the library writes it
        fill = bytes([2, 3 if chunked else 2, 2, 1]) + struct.pack("<I", 0)
        msgs = [(M_DATASPACE, _dataspace_msg(a.shape), 0), (M_DATATYPE, _dtype_msg(a.dtype), 1),
                (M_FILL, fill, 1)]
        raw = a.tobytes()
        if chunked:
            cshape = tuple(int(c) for c in chunks[k.decode("utf-8")])
            if len(cshape) != a.ndim or a.ndim == 0 or any(c < 1 or c > d for c, d in zip(cshape, a.shape)):
                raise ValueError(f"{k!r}: chunk shape {cshape} for an array of shape {a.shape}")
            grid = [range(0, d, c) for d, c in zip(a.shape, cshape)]
            origins = np.stack(np.meshgrid(*grid, indexing="ij"), -1).reshape(-1, a.ndim)
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
                msgs.append((M_FILTERS, fm, 0))
            def encode(o, a=a, cshape=cshape, pipe=pipe):
                sl = tuple(slice(int(s), int(s) + c) for s, c in zip(o, cshape))
                c = np.zeros(cshape, a.dtype)
                part = a[sl]
                c[tuple(slice(0, n) for n in part.shape)] = part
                d = c.tobytes()
                for fid, cd in pipe:
                    d = _shuffle(d, cd[0]) if fid == F_SHUFFLE else zlib.compress(d, cd[0])
                return d

            data = _parallel_map(encode, list(origins))
            dims4 = b"".join(struct.pack("<I", c) for c in cshape + (a.itemsize,))
            v4 = bytes([4, 2])
            if new_format and len(origins) == 1:  # layout v4, single-chunk index
                addr = al.take(len(data[0]))
                al.put(addr, data[0])
                lay = v4 + bytes([2 if pipe else 0, a.ndim + 1, 4]) + dims4 + bytes([1])
                if pipe:
                    lay += struct.pack("<QI", len(data[0]), 0)
                lay += struct.pack("<Q", addr)
            elif new_format and not pipe:  # layout v4, implicit index: full chunks in grid order
                addr = al.take(sum(len(d) for d in data))
                al.put(addr, b"".join(data))
                lay = v4 + bytes([0, a.ndim + 1, 4]) + dims4 + bytes([2]) + struct.pack("<Q", addr)
            else:  # layout v3, v1 B-tree chunk index of one leaf
                if len(origins) > 2 * ISTORE_K:
                    raise ValueError(f"{k!r}: {len(origins)} chunks (at most {2 * ISTORE_K} are written)")
                nd = a.ndim + 1
                ks = 8 + 8 * nd
                node_size = 24 + (2 * ISTORE_K + 1) * ks + 2 * ISTORE_K * 8
                btree = al.take(node_size)
                node = bytearray(b"TREE" + bytes([1, 0]) + struct.pack("<HQQ", len(origins), UNDEF, UNDEF))
                for o, d in zip(origins, data):
                    addr = al.take(len(d))
                    al.put(addr, d)
                    node += struct.pack("<II", len(d), 0) + b"".join(struct.pack("<Q", int(v)) for v in o)
                    node += struct.pack("<Q", 0) + struct.pack("<Q", addr)
                # the final key: the last chunk's offset plus the chunk dimensions
                node += struct.pack("<II", 0, 0) + b"".join(
                    struct.pack("<Q", int(o) + c) for o, c in zip(origins[-1], cshape)) + struct.pack("<Q", 0)
                node += b"\0" * (node_size - len(node))
                al.put(btree, bytes(node))
                lay = bytes([3, 2, nd]) + struct.pack("<Q", btree) + dims4
        else:
            addr = al.take(len(raw)) if raw else UNDEF
            if raw:
                al.put(addr, raw)
            lay = bytes([3, 1]) + struct.pack("<QQ", addr, len(raw))
        msgs.append((M_LAYOUT, lay, 0))
        oh = _object_header(msgs, new_format)
        oh_addr = al.take(len(oh))
        al.put(oh_addr, oh)
        entries.append((k, oh_addr))

    if links:
        if len(entries) > MAX_COMPACT_LINKS:
            heap, names = _dense_links(al, entries)
            rmsgs = [(M_LINK_INFO, bytes([0, 0]) + struct.pack("<QQ", heap, names), 0)]
        else:
            rmsgs = [(M_LINK_INFO, bytes([0, 0]) + struct.pack("<QQ", UNDEF, UNDEF), 0)]
        rmsgs.append((M_GROUP_INFO, bytes([0, 0]), 0))
        if len(entries) <= MAX_COMPACT_LINKS:
            rmsgs += [(M_LINK, _link_msg(k, a), 0) for k, a in entries]
        root = _object_header(rmsgs, new_format)
        root_addr = al.take(len(root))
        al.put(root_addr, root)
        root_entry = struct.pack("<QQI4x", 0, root_addr, 0) + b"\0" * 16  # no cached group data
    else:
        root_addr, root_entry = _symbol_table_root(al, entries, new_format)
    eof = al.end
    if new_format:
        sb = SIG + bytes([2, 8, 8, 0]) + struct.pack("<QQQQ", 0, UNDEF, eof, root_addr)
        sb += struct.pack("<I", lookup3(sb))
    else:
        sb = (SIG + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", GROUP_LEAF_K, GROUP_INTERNAL_K, 0)
              + struct.pack("<QQQQ", 0, UNDEF, eof, UNDEF) + root_entry)
        assert len(sb) == 96
    with open(path, "wb") as f:
        f.write(sb)
        pos = len(sb)
        for addr, data in sorted(al.blocks, key=lambda x: x[0]):
            if addr > pos:
                f.write(b"\0" * (addr - pos))
            f.write(data)
            pos = addr + len(data)
        if eof > pos:
            f.write(b"\0" * (eof - pos))
    return path


def _symbol_table_root(al: _Alloc, entries: list, v2: bool) -> tuple[int, bytes]:
    """The root group as a symbol table: a local heap of the names ("" at 0, each name
    NUL-terminated on an 8-byte grid, then a free block), symbol-table nodes of up to 2K
    entries and one leaf of the group B-tree. Returns (object header address, superblock
    root entry with the B-tree and heap cached)."""
    heap_data, name_off = bytearray(8), {}
    for k, _ in entries:
        name_off[k] = len(heap_data)
        heap_data += k + b"\0" * (_pad8(len(k) + 1) - len(k))
    free_off = len(heap_data)
    heap_data += struct.pack("<QQ", HEAP_FREE_NULL, 16)  # one free block of 16 bytes (next: none)
    heap_hdr, heap_seg = al.take(32), al.take(len(heap_data))
    al.put(heap_hdr, b"HEAP" + b"\0" * 4 + struct.pack("<QQQ", len(heap_data), free_off, heap_seg))
    al.put(heap_seg, bytes(heap_data))
    cap = 2 * GROUP_LEAF_K
    snods = [entries[i:i + cap] for i in range(0, len(entries), cap)]
    if len(snods) > 2 * GROUP_INTERNAL_K:
        raise ValueError(f"{len(entries)} datasets (at most {2 * GROUP_INTERNAL_K * cap} are written)")
    snod_size = 8 + cap * 40
    node_size = 24 + (2 * GROUP_INTERNAL_K + 1) * 8 + 2 * GROUP_INTERNAL_K * 8
    btree = al.take(node_size)
    node = bytearray(b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", len(snods), UNDEF, UNDEF))
    node += struct.pack("<Q", 0)  # key 0: the empty name
    for s in snods:
        sa = al.take(snod_size)
        body = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(s)))
        for k, oh in s:
            body += struct.pack("<QQI4x", name_off[k], oh, 0) + b"\0" * 16
        body += b"\0" * (snod_size - len(body))
        al.put(sa, bytes(body))
        node += struct.pack("<Q", sa) + struct.pack("<Q", name_off[s[-1][0]])
    node += b"\0" * (node_size - len(node))
    al.put(btree, bytes(node))
    root = _object_header([(M_SYMBOL_TABLE, struct.pack("<QQ", btree, heap_hdr), 0)], v2)
    root_addr = al.take(len(root))
    al.put(root_addr, root)
    return root_addr, struct.pack("<QQI4x", 0, root_addr, 1) + struct.pack("<QQ", btree, heap_hdr)
