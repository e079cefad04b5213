"""VTK structured grids: the debug output of the primitive state (IO.jl:213-233,
debugOutput) and the set-up scripts' mesh.vts (parse_mesh.jl:275-289, readfort.jl:237-239).

The reference writes rho, u, v, w, p, T of every cell, ghosts included, at the ghost-filled
cell-centre coordinates, with WriteVTK's `vtk_grid`: an XML StructuredGrid file (.vts).
`write_debug_vts` writes the same grid and point arrays in VTK's XML format (Float32, one
appended raw block per array, each preceded by its UInt64 byte count); `read_vts` reads
such a file back. Arrays are in the reference layout seen from C order: Q (6, Nz+8, Ny+8,
Nx+8), coordinates (Nz+8, Ny+8, Nx+8); VTK's point order (x fastest) is that memory order.
"""
from __future__ import annotations

import re
import xml.etree.ElementTree as ET

import numpy as np

NAMES = ("rho", "u", "v", "w", "p", "T")


def write_vts(path: str, x: np.ndarray, y: np.ndarray, z: np.ndarray, arrays: dict) -> str:
    """Write the named point arrays (each of x's shape) at the points (x, y, z) to `path`
    (.vts, appended raw Float32 blocks), as WriteVTK's vtk_grid does."""
    if y.shape != x.shape or z.shape != x.shape or x.ndim != 3:
        raise ValueError("x, y, z must be 3-D arrays of one shape")
    if any(np.shape(a) != x.shape for a in arrays.values()):
        raise ValueError("every point array needs the shape of x")
    nz, ny, nx = x.shape
    if not path.endswith(".vts"):
        path += ".vts"
    extent = f"0 {nx - 1} 0 {ny - 1} 0 {nz - 1}"
    blocks, offsets, off = [], [], 0
    pts = np.stack([np.asarray(a, dtype="<f4").ravel() for a in (x, y, z)], axis=1).ravel()
    for arr in [pts] + [np.asarray(a, dtype="<f4").ravel() for a in arrays.values()]:
        raw = arr.tobytes()
        blocks.append(np.array([len(raw)], dtype="<u8").tobytes() + raw)
        offsets.append(off)
        off += len(blocks[-1])
    head = ['<?xml version="1.0"?>',
            '<VTKFile type="StructuredGrid" version="1.0" byte_order="LittleEndian" header_type="UInt64">',
            f'  <StructuredGrid WholeExtent="{extent}">',
            f'    <Piece Extent="{extent}">',
            '      <PointData>']
    for n, name in enumerate(arrays):
        head.append(f'        <DataArray type="Float32" Name="{name}" NumberOfComponents="1" '
                    f'format="appended" offset="{offsets[n + 1]}"/>')
    head += ['      </PointData>',
             '      <Points>',
             f'        <DataArray type="Float32" Name="Points" NumberOfComponents="3" format="appended" '
             f'offset="{offsets[0]}"/>',
             '      </Points>',
             '    </Piece>',
             '  </StructuredGrid>',
             '  <AppendedData encoding="raw">']
    with open(path, "wb") as f:
        f.write(("\n".join(head) + "\n   _").encode())
        for b in blocks:
            f.write(b)
        f.write(b"\n  </AppendedData>\n</VTKFile>\n")
    return path


def write_debug_vts(path: str, Q: np.ndarray, x: np.ndarray, y: np.ndarray, z: np.ndarray) -> str:
    """Write Q's six primitive variables at the points (x, y, z) to `path` (.vts appended)."""
    Q = np.asarray(Q)
    if Q.ndim != 4 or Q.shape[0] != 6 or x.shape != Q.shape[1:]:
        raise ValueError("Q must be (6, Nz, Ny, Nx) and x, y, z (Nz, Ny, Nx)")
    return write_vts(path, x, y, z, {name: Q[n] for n, name in enumerate(NAMES)})


# parse_mesh.jl:275-289 names the metrics dkdx ... dsdz (xi, eta, zeta as k, e, s)
MESH_METRIC_NAMES = ("dkdx", "dkdy", "dkdz", "dedx", "dedy", "dedz", "dsdx", "dsdy", "dsdz")


def write_mesh_vts(path: str, x, y, z, J, metrics=None) -> str:
    """mesh.vts of the reference's set-up scripts: J at every grid point with ghosts, and the
    nine metrics as parse_mesh.jl:275-289 adds them (readfort.jl:237-239 writes J only)."""
    arrays = {"J": J}
    if metrics is not None:
        arrays.update(zip(MESH_METRIC_NAMES, metrics))
    return write_vts(path, np.asarray(x), np.asarray(y), np.asarray(z), arrays)


def read_vts(path: str) -> dict:
    """{'extent': (nx, ny, nz), 'points': (N, 3), name: (N,) ...} from a file of write_debug_vts."""
    data = open(path, "rb").read()
    mark = data.index(b"<AppendedData")
    start = data.index(b"_", mark) + 1
    xml = re.sub(r"<\?xml[^>]*\?>", "", data[:mark].decode()) + "</VTKFile>"  # close the root
    root = ET.fromstring(xml)
    piece = root.find("StructuredGrid/Piece")
    e = [int(v) for v in piece.get("Extent").split()]
    out = {"extent": (e[1] + 1, e[3] + 1, e[5] + 1)}

    def block(offset: int, ncomp: int) -> np.ndarray:
        p = start + offset
        nbytes = int(np.frombuffer(data[p:p + 8], dtype="<u8")[0])
        a = np.frombuffer(data[p + 8:p + 8 + nbytes], dtype="<f4")
        return a.reshape(-1, ncomp) if ncomp > 1 else a

    for da in piece.iter("DataArray"):
        out["points" if da.get("Name") == "Points" else da.get("Name")] = block(
            int(da.get("offset")), int(da.get("NumberOfComponents")))
    return out
