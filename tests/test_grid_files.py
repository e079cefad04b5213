"""The mesh file of the reference's grid generator (OCFD3d-Mesh.dat, Fortran unformatted
records written by SCU-benchmark/swept-compression-ramp.c:451-560) and readfort.jl's reading
of it (:14-100): byte layout, round trip, damaged-file detection, and the Float32 ghost
extension and unit conversion against a loop restatement of readfort.jl. Bitwise checks
(integer layout; the same IEEE float32 operations in the same order)."""
import numpy as np
import pytest

from flame3d_mhd_gb300.grid import NG, compression_ramp_grid, mesh_from_ocfd, read_ocfd_mesh, write_ocfd_mesh
from test_grid import _readfort_loops


def _interior(nx=6, ny=5, nz=3, seed=1):
    rng = np.random.default_rng(seed)
    return tuple(rng.standard_normal((nz, ny, nx)) * 10 for _ in range(3))


def test_record_layout(tmp_path):
    x, y, z = _interior()
    p = tmp_path / "OCFD3d-Mesh.dat"
    write_ocfd_mesh(str(p), x, y, z)
    raw = p.read_bytes()
    nz, ny, nx = x.shape
    rec = nx * ny * 8
    assert len(raw) == 3 * nz * (rec + 8)
    assert np.frombuffer(raw[:4], "<i4")[0] == rec
    assert np.frombuffer(raw[4:4 + rec], "<f8").reshape(ny, nx).tolist() == x[0].tolist()
    assert np.frombuffer(raw[4 + rec:8 + rec], "<i4")[0] == rec
    # the y planes start after the nz x records
    off = nz * (rec + 8)
    assert np.frombuffer(raw[off + 4:off + 12], "<f8")[0] == y[0, 0, 0]


def test_round_trip_and_damage(tmp_path):
    x, y, z = _interior()
    p = tmp_path / "m.dat"
    write_ocfd_mesh(str(p), x, y, z)
    nz, ny, nx = x.shape
    xr, yr, zr = read_ocfd_mesh(str(p), nx, ny, nz)
    assert np.array_equal(xr, x) and np.array_equal(yr, y) and np.array_equal(zr, z)
    with pytest.raises(ValueError):
        read_ocfd_mesh(str(p), nx + 1, ny, nz)
    raw = bytearray(p.read_bytes())
    raw[0] ^= 1  # damage the first record marker
    q = tmp_path / "bad.dat"
    q.write_bytes(bytes(raw))
    with pytest.raises(ValueError):
        read_ocfd_mesh(str(q), nx, ny, nz)
    q.write_bytes(bytes(raw[:-3]))
    with pytest.raises(ValueError):
        read_ocfd_mesh(str(q), nx, ny, nz)


def test_generate_xyz_float32_matches_readfort(tmp_path):
    nx, ny, nz = 12, 8, 6
    x, y, z, _ = compression_ramp_grid(nx, ny, nz, first_cell=1e-2)
    I = (slice(NG, NG + nz), slice(NG, NG + ny), slice(NG, NG + nx))
    xm, ym, zm = (a[I] * 1000.0 for a in (x, y, z))  # the generator's millimetres
    p = tmp_path / "OCFD3d-Mesh.dat"
    write_ocfd_mesh(str(p), xm, ym, zm)
    X, Y, Z = mesh_from_ocfd(str(p), nx, ny, nz)
    # readfort.jl: Float32 arrays, its ghost loops in Float32, then ./= 1000.f0
    ref = []
    for a in (xm, ym, zm):
        A = np.zeros(X.shape, dtype=np.float32)
        A[I] = a.astype(np.float32)
        ref.append(A)
    R = _readfort_loops(*(A.T.copy() for A in ref))  # Julia (i, j, k) order
    for got, want in zip((X, Y, Z), R):
        assert got.dtype == np.float32 and want.dtype == np.float32
        assert np.array_equal(got, want.T / np.float32(1000.0))
    # FP64 path: the file's doubles, the ghost extension in FP64, metres
    X64, Y64, Z64 = mesh_from_ocfd(str(p), nx, ny, nz, dtype=np.float64)
    assert np.abs(X64 - x).max() <= 1e-12 * np.abs(x).max()
    assert np.abs(Y64 - y).max() <= 1e-12 * np.abs(y).max()
