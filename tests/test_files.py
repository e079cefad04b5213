"""The reference's HDF5 files without an HDF5 library (CPU).

The reader is pinned on a file that the HDF5 library itself wrote (a MATLAB 7.3 file that
SciPy ships as a test fixture: a 512-byte user block, a version-0 superblock, a symbol-table
root group, one contiguous float64 dataset with a string attribute); the writer's message
encodings are compared byte for byte with that file's, its structures are checked against
the rules the library enforces on reading (end-of-file address, B-tree and symbol-table node
capacities and keys, the local heap's free list, 8-byte message alignment), and every file
kind round-trips through the reader. The IO.jl / parse_mesh.jl wrappers are checked for
names, shapes, Float32 values and the solver's ghost extrapolation.
"""
import os
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from flame3d_mhd_gb300 import files, h5
from flame3d_mhd_gb300.grid import NG, extend_ghosts

FIXTURE = None
try:
    import scipy.io.matlab as _sm

    FIXTURE = os.path.join(os.path.dirname(_sm.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
except ImportError:
    pass


def _fixture():
    if FIXTURE is None or not os.path.exists(FIXTURE):
        pytest.skip("SciPy's HDF5 test file is not installed")
    return FIXTURE


def test_reader_on_a_file_written_by_the_hdf5_library():
    with h5.H5File(_fixture()) as f:
        assert f.base == 512  # the user block
        assert f.keys() == ["testdouble"]
        d = f.dataset("testdouble")
        assert d.shape == (9, 1) and d.dtype == np.dtype("<f8") and d.layout[0] == "contiguous"
        assert d.attrs == {"MATLAB_class": "double"}
        assert np.array_equal(d.read()[:, 0], np.linspace(0, 2 * np.pi, 9))


def test_writer_messages_match_the_library_encoding():
    with h5.H5File(_fixture()) as f:
        msgs = dict(f.messages(f.group()["testdouble"]))
    # message bodies as stored: padded to 8 bytes
    assert h5._message(h5.M_DATATYPE, h5._dtype_msg(np.dtype("<f8")))[8:] == msgs[h5.M_DATATYPE]
    assert h5._message(h5.M_DATASPACE, h5._dataspace_msg((9, 1)))[8:] == msgs[h5.M_DATASPACE]


def _structure_checks(path):
    """The checks the HDF5 library makes when it opens the file and its root group."""
    raw = open(path, "rb").read()
    with h5.H5File(path) as f:
        assert f.eof == len(raw) and f.base == 0
        b = f.buf
        # root entry's cached B-tree and heap equal the symbol-table message
        st = dict(f.messages(f.root[1]))[h5.M_SYMBOL_TABLE]
        assert f.root[2] == 1 and f.root[3] == st
        btree, heap = struct.unpack("<QQ", st)
        # local heap: "" at 0, the free list inside the segment, ending at 1
        assert b[heap:heap + 4] == b"HEAP"
        size, free, data = struct.unpack("<QQQ", b[heap + 8:heap + 32])
        assert b[data:data + 8] == b"\0" * 8 and size % 8 == 0
        nxt, fsize = struct.unpack("<QQ", b[data + free:data + free + 16])
        assert nxt == h5.HEAP_FREE_NULL and free + fsize <= size and fsize >= 16
        # group B-tree: at most 2K children, keys bracket the names of each symbol-table node
        assert b[btree:btree + 6] == b"TREE\0\0"
        used = struct.unpack("<H", b[btree + 6:btree + 8])[0]
        assert used <= 2 * h5.GROUP_INTERNAL_K
        name = lambda off: bytes(b[data + off:b.find(b"\0", data + off)])
        prev_key = name(struct.unpack("<Q", b[btree + 24:btree + 32])[0])
        assert prev_key == b""
        p = btree + 32
        for _ in range(used):
            snod, key = struct.unpack("<QQ", b[p:p + 16])
            p += 16
            assert b[snod:snod + 6] == b"SNOD\x01\0"
            n = struct.unpack("<H", b[snod + 6:snod + 8])[0]
            assert 0 < n <= 2 * h5.GROUP_LEAF_K
            names = [name(struct.unpack("<Q", b[snod + 8 + 40 * i:snod + 16 + 40 * i])[0]) for i in range(n)]
            assert names == sorted(names) and prev_key < names[0] and names[-1] == name(key)
            prev_key = name(key)
            # each dataset header: version 1, message count, 8-byte aligned messages filling the size
            for i in range(n):
                oh = struct.unpack("<Q", b[snod + 16 + 40 * i:snod + 24 + 40 * i])[0]
                ver, nmsg, refc, hsize = struct.unpack("<BxHII", b[oh:oh + 12])
                assert ver == 1 and refc == 1 and hsize % 8 == 0
                q, count = oh + 16, 0
                while q < oh + 16 + hsize:
                    msize = struct.unpack("<H", b[q + 2:q + 4])[0]
                    assert msize % 8 == 0
                    q += 8 + msize
                    count += 1
                assert q == oh + 16 + hsize and count == nmsg


def test_round_trip_types_shapes_and_many_names(tmp_path):
    rng = np.random.default_rng(0)
    d = {"dξdx": rng.standard_normal((5, 6, 7)).astype(np.float32), "J": rng.standard_normal((5, 6, 7)),
         "NG": np.int64(4), "Nx": 7, "u8": np.arange(5, dtype=np.uint8), "i16": -np.arange(3, dtype=np.int16),
         "coords": np.ascontiguousarray(rng.standard_normal((3, 4, 5, 3)).astype(np.float32)[:, ::-1]),
         "empty": np.zeros((0, 3))}
    for i in range(23):  # three symbol-table nodes
        d[f"x{i:02d}"] = np.arange(i + 1, dtype=np.int32)
    p = h5.write(str(tmp_path / "t.h5"), d)
    _structure_checks(p)
    r = h5.read(p)
    assert sorted(r) == sorted(d)
    for k, v in d.items():
        v = np.asarray(v)
        assert r[k].dtype == v.dtype and r[k].shape == v.shape and np.array_equal(r[k], v), k
    # an empty file
    p = h5.write(str(tmp_path / "e.h5"), {})
    _structure_checks(p)
    assert h5.read(p) == {}


@pytest.mark.parametrize("deflate,shuffle", [(None, False), (None, True), (1, True), (6, False)])
def test_chunked_round_trip(tmp_path, deflate, shuffle):
    rng = np.random.default_rng(1)
    a = rng.standard_normal((9, 10, 11)).astype(np.float32)
    b = rng.standard_normal((2, 6, 5, 4, 3))
    p = h5.write(str(tmp_path / "c.h5"), {"a": a, "b": b}, chunks={"a": (4, 5, 6), "b": (1, 6, 5, 4, 3)},
                 deflate=deflate, shuffle=shuffle)
    _structure_checks(p)
    with h5.H5File(p) as f:
        da = f.dataset("a")
        assert da.layout[0] == "chunked" and da.layout[2] == [4, 5, 6, 4]
        assert [fid for fid, _ in da.filters] == ([h5.F_SHUFFLE] if shuffle else []) + \
            ([h5.F_DEFLATE] if deflate is not None else [])
        assert len(list(f.chunk_entries(da.layout[1], 4))) == 3 * 2 * 2  # ragged edge chunks
        assert np.array_equal(f["a"], a) and np.array_equal(f["b"], b)


def test_writer_and_reader_errors(tmp_path):
    a = np.zeros((130, 2), np.float32)
    with pytest.raises(ValueError):
        h5.write(str(tmp_path / "x.h5"), {"a": a}, chunks={"a": (1, 2)})  # 130 chunks
    with pytest.raises(ValueError):
        h5.write(str(tmp_path / "x.h5"), {"a": a}, chunks={"a": (200, 2)})  # chunk larger than the array
    with pytest.raises(ValueError):
        h5.write(str(tmp_path / "x.h5"), {"g/a": a})
    with pytest.raises(ValueError):
        h5.write(str(tmp_path / "x.h5"), {"a": np.zeros(2, np.complex64)})
    p = tmp_path / "not.h5"
    p.write_bytes(b"plain text, no signature" * 40)
    with pytest.raises(ValueError):
        h5.H5File(str(p))
    good = h5.write(str(tmp_path / "g.h5"), {"a": a})
    raw = bytearray(open(good, "rb").read())
    raw[8] = 2  # a superblock of the newer format
    (tmp_path / "v2.h5").write_bytes(bytes(raw))
    with pytest.raises(ValueError):
        h5.H5File(str(tmp_path / "v2.h5"))
    with h5.H5File(good) as f:
        with pytest.raises(KeyError):
            f["b"]


def _grid(n=(6, 5, 7), seed=2):
    rng = np.random.default_rng(seed)
    nz, ny, nx = n
    shape = (nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)
    k, j, i = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
    x = i * 0.1 + 0.01 * np.sin(j)
    y = j * 0.2 + 0.02 * np.cos(i + k)
    z = k * 0.3 + 0.01 * rng.standard_normal(shape)
    return x, y, z


def test_metrics_and_mesh_files(tmp_path):
    rng = np.random.default_rng(3)
    shape = (6 + 2 * NG, 5 + 2 * NG, 7 + 2 * NG)
    m = [rng.standard_normal(shape) for _ in range(9)]
    J = rng.random(shape) + 0.5
    for compress in (3, None):
        p = files.write_metrics(str(tmp_path / f"metrics{compress}.h5"), m, J, compress=compress)
        _structure_checks(p)
        with h5.H5File(p) as f:
            assert f.keys() == sorted(files.METRIC_NAMES + ("J",), key=lambda s: s.encode())
            assert all(f.dataset(k).dtype == np.float32 for k in f.keys())
            assert (f.dataset("J").layout[0] == "chunked") == (compress is not None)
        m2, J2 = files.read_metrics(p)
        assert all(np.array_equal(a, b.astype(np.float32).astype(np.float64)) for a, b in zip(m2, m))
        assert np.array_equal(J2, J.astype(np.float32))
    x, y, z = _grid()
    p = files.write_mesh(str(tmp_path / "mesh.h5"), x, y, z)
    _structure_checks(p)
    with h5.H5File(p) as f:
        assert [int(f[k]) for k in ("NG", "Nx", "Ny", "Nz")] == [NG, 7, 5, 6]
        assert f.dataset("NG").shape == () and f.dataset("NG").dtype == np.int64
        c = f["coords"]
    assert c.shape == (6, 5, 7, 3) and c.dtype == np.float32
    assert np.array_equal(c[..., 1], y[NG:-NG, NG:-NG, NG:-NG].astype(np.float32))
    # read back: interior as written, ghosts by the solver's extrapolation in Float32
    X, Y, Z = files.read_mesh(p)
    ref = extend_ghosts(*[np.pad(a[NG:-NG, NG:-NG, NG:-NG].astype(np.float32), NG) for a in (x, y, z)],
                        dtype=np.float32, rule="solver")
    for A, R in zip((X, Y, Z), ref):
        assert A.dtype == np.float32 and np.array_equal(A, R)


def test_solution_files(tmp_path):
    rng = np.random.default_rng(4)
    nz, ny, nx = 6, 5, 7
    Q = rng.standard_normal((6, nz + 2 * NG, ny + 2 * NG, nx + 2 * NG))
    phi = rng.random((nz + 2 * NG, ny + 2 * NG, nx + 2 * NG))
    I = (slice(NG, -NG),) * 3
    out = str(tmp_path)
    p = files.plotFile_xdmf(out, 500, Q, phi, dt=2e-3)
    assert p == os.path.join(out, "PLT", "plt-500.h5")
    _structure_checks(p)
    r = h5.read(p)
    assert sorted(r) == sorted(files.PRIM_NAMES + ("phi",))
    for n, name in enumerate(files.PRIM_NAMES):
        assert np.array_equal(r[name], Q[n][I].astype(np.float32))
    assert np.array_equal(r["phi"], phi[I].astype(np.float32))
    # the XDMF file: time, topology and every attribute pointing at a dataset of its dimensions
    root = ET.parse(os.path.join(out, "PLT", "plt-500.xmf")).getroot()
    grid = root.find("Domain/Grid")
    assert float(grid.find("Time").get("Value")) == pytest.approx(1.0)
    assert grid.find("Topology").get("NumberOfElements") == f"{nz} {ny} {nx}"
    assert grid.find("Geometry/DataItem").get("Dimensions") == f"{nz} {ny} {nx} 3"
    names = []
    for att in grid.findall("Attribute"):
        item = att.find("DataItem")
        fname, dset = item.text.strip().split(":/")
        assert fname == "plt-500.h5" and r[dset].shape == tuple(int(v) for v in item.get("Dimensions").split())
        names.append(att.get("Name"))
    assert names == list(files.PRIM_NAMES) + ["phi"]

    p = files.plotFile_h5(out, 600, Q, compress=None)
    assert np.array_equal(h5.read(p)["Q"], Q[(slice(None),) + I].astype(np.float32))
    p = files.checkpointFile(out, 700, Q)
    _structure_checks(p)
    with h5.H5File(p) as f:
        d = f.dataset("Q_h")
        assert d.shape == (1,) + Q.shape and d.layout[2][:5] == [1, 1] + list(Q.shape[1:])  # a chunk a variable
        assert [fid for fid, _ in d.filters] == [h5.F_SHUFFLE, h5.F_DEFLATE]
    assert np.array_equal(files.read_checkpoint(p), Q.astype(np.float32))
    p = files.averageFile(out, 800, Q)
    assert np.array_equal(h5.read(p)["avg"], Q[(slice(None),) + I].astype(np.float32))


def test_lookup3_published_vectors():
    # Bob Jenkins' lookup3.c driver values for hashlittle
    s = b"Four score and seven years ago"
    assert h5.lookup3(b"", 0) == 0xDEADBEEF
    assert h5.lookup3(b"", 0xDEADBEEF) == 0xBD5B7DDE
    assert h5.lookup3(s, 0) == 0x17770551
    assert h5.lookup3(s, 1) == 0xCD628161


@pytest.mark.parametrize("new_format", [False, True])
@pytest.mark.parametrize("links,n", [(False, 3), (True, 3), (True, 12)])
def test_link_groups_and_version2_headers(tmp_path, new_format, links, n):
    """Groups as link messages (compact, and dense in a fractal heap indexed by link-name
    hashes), version-2 superblock and object headers, the single-chunk and implicit chunk
    indexes; every checksum is verified on reading."""
    rng = np.random.default_rng(5)
    d = {f"dξd{i:02d}": rng.standard_normal((3, 4, 5)).astype(np.float32) for i in range(n)}
    d.update(NG=np.int64(4), Q=rng.standard_normal((6, 5, 4, 3)), c=rng.standard_normal((9, 10, 11)),
             e=rng.standard_normal((9, 10, 11)).astype(np.float32))
    p = h5.write(str(tmp_path / "n.h5"), d, chunks={"Q": (6, 5, 4, 3), "c": (4, 5, 6), "e": (4, 5, 6)},
                 links=links, new_format=new_format)
    with h5.H5File(p) as f:
        assert f.version == (2 if new_format else 0) and f.eof == os.path.getsize(p)
        msgs = dict(f.messages(f.root[1]))
        if links:
            heap = struct.unpack("<Q", msgs[h5.M_LINK_INFO][2:10])[0]
            assert (heap != h5.UNDEF) == (len(d) > h5.MAX_COMPACT_LINKS)
        else:
            assert h5.M_SYMBOL_TABLE in msgs
        kinds = {k: f.dataset(k).layout[0] for k in ("Q", "c")}
        assert kinds == ({"Q": "single", "c": "implicit"} if new_format else {"Q": "chunked", "c": "chunked"})
        r = {k: f[k] for k in f.keys()}
    assert sorted(r) == sorted(d)
    for k, v in d.items():
        assert np.array_equal(r[k], np.asarray(v)), k
    # filtered: single chunk with its filtered size, several chunks through the v1 B-tree
    p = h5.write(str(tmp_path / "z.h5"), d, chunks={"Q": (6, 5, 4, 3), "c": (4, 5, 6)}, deflate=3, shuffle=True,
                 links=links, new_format=new_format)
    with h5.H5File(p) as f:
        assert f.dataset("c").layout[0] == "chunked"
        assert f.dataset("Q").layout[0] == ("single" if new_format else "chunked")
        assert np.array_equal(f["Q"], d["Q"]) and np.array_equal(f["c"], d["c"])


def test_checksums_catch_damage(tmp_path):
    d = {f"x{i:02d}": np.arange(i + 2, dtype=np.float64) for i in range(12)}
    p = h5.write(str(tmp_path / "d.h5"), d, links=True, new_format=True)
    raw = open(p, "rb").read()
    with h5.H5File(p) as f:
        assert f.keys() == sorted(d, key=lambda s: h5.lookup3(s.encode()))  # the name index's hash order
    for sig in (b"OHDR", b"FRHP", b"BTHD", b"BTLF"):
        bad = bytearray(raw)
        at = raw.index(sig) + 6
        bad[at] ^= 0x40
        q = tmp_path / "bad.h5"
        q.write_bytes(bytes(bad))
        with pytest.raises(ValueError):
            with h5.H5File(str(q)) as f:
                [f[k] for k in f.keys()]
    bad = bytearray(raw)
    bad[20] ^= 1  # inside the version-2 superblock
    (tmp_path / "sb.h5").write_bytes(bytes(bad))
    with pytest.raises(ValueError):
        h5.H5File(str(tmp_path / "sb.h5"))


# Cartesian coordinates of each rank of MPI_Cart_create (run.jl:117 with reorder off), written
# out from the MPI standard's rule (ranks in row-major order of the coordinates, the last
# dimension varying fastest) rather than computed, so a wrong ordering in assemble_checkpoint
# cannot cancel against the same mistake here.
CART_COORDS = {
    (1, 1, 1): [(0, 0, 0)],
    (2, 1, 1): [(0, 0, 0), (1, 0, 0)],
    (2, 3, 2): [(0, 0, 0), (0, 0, 1), (0, 1, 0), (0, 1, 1), (0, 2, 0), (0, 2, 1),
                (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1), (1, 2, 0), (1, 2, 1)],
}


@pytest.mark.parametrize("nprocs", [(1, 1, 1), (2, 1, 1), (2, 3, 2)])
def test_assemble_multi_rank_checkpoint(tmp_path, nprocs):
    """Blocks cut from a global field with their ghost frames, as each rank of a multi-GPU
    run holds them, reassemble to that field."""
    px, py, pz = nprocs
    nxp, nyp, nzp = 5, 4, 3
    rng = np.random.default_rng(8)
    G0 = rng.standard_normal((6, pz * nzp + 2 * NG, py * nyp + 2 * NG, px * nxp + 2 * NG)).astype(np.float32)
    blocks = []
    for r in range(px * py * pz):
        cx, cy, cz = CART_COORDS[nprocs][r]
        blocks.append(G0[:, cz * nzp:(cz + 1) * nzp + 2 * NG, cy * nyp:(cy + 1) * nyp + 2 * NG,
                         cx * nxp:(cx + 1) * nxp + 2 * NG])
    p = h5.write(str(tmp_path / "chk.h5"), {"Q_h": np.stack(blocks)})
    assert np.array_equal(files.assemble_checkpoint(p, nprocs), G0)
    with pytest.raises(ValueError):
        files.assemble_checkpoint(p, (px * py * pz + 1, 1, 1))
