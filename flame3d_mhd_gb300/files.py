"""The reference's on-disk files, written and read through `h5` (no HDF5 library needed):

  metrics.h5   nine metrics and J, Float32 with ghosts     parse_mesh.jl:250-261, solver.jl:237-250
  mesh.h5      NG, Nx, Ny, Nz and the interior coords      parse_mesh.jl:262-273, solver.jl:252-274
  PLT/plt-tt.h5 + .xmf   rho u v w p T phi, interior        IO.jl:1-112 (plotFile_xdmf), 236-292
  PLT/plt-tt.h5 (Q)      the six primitives, interior       IO.jl:114-151 (plotFile_h5)
  CHK/chk-tt.h5 (Q_h)    the primitives with ghosts, by rank IO.jl:153-183, solver.jl:211-216
  AVG/avg-tt.h5 (avg)    averaged primitives, interior       IO.jl:185-210

Layouts: this package's arrays are the reference's Julia arrays seen from C order, and
HDF5.jl writes a Julia array with its dimensions reversed, so the datasets carry this
package's shapes: a metric is (Nz+8, Ny+8, Nx+8), coords (Nz, Ny, Nx, 3) (Julia (3, Nx, Ny,
Nz)), Q_h (ranks, 6, Nz+8, Ny+8, Nx+8) (Julia (Nx+8, Ny+8, Nz+8, 6, ranks)). Values are
Float32 as the reference writes them. Arrays may be numpy arrays or torch tensors (copied to
the host). The reference compresses with shuffle + deflate (levels from run.jl:30-43,
parse_mesh.jl:17); `compress=None` writes contiguous, uncompressed datasets instead.
"""
from __future__ import annotations

import os

import numpy as np

from . import h5
from .grid import NG, extend_ghosts

METRIC_NAMES = ("dξdx", "dξdy", "dξdz", "dηdx", "dηdy", "dηdz", "dζdx", "dζdy", "dζdz")
PRIM_NAMES = ("rho", "u", "v", "w", "p", "T")
MAX_CHUNKS = 2 * h5.ISTORE_K


def _host(a, dtype=np.float32) -> np.ndarray:
    if hasattr(a, "detach"):
        a = a.detach().cpu().numpy()
    return np.asarray(a, dtype=dtype)


def _interior(a: np.ndarray) -> np.ndarray:
    return a[..., NG:-NG, NG:-NG, NG:-NG]


def _slabs(shape) -> tuple:
    """A chunk shape that splits `shape` into at most MAX_CHUNKS slabs along its slowest
    axis longer than 1 (the chunks are compressed in parallel; readers see no difference
    from the reference's one chunk a rank)."""
    axis = next((d for d, n in enumerate(shape) if n > 1), 0)
    c = list(shape)
    c[axis] = max(1, -(-shape[axis] // MAX_CHUNKS))
    return tuple(c)


def _write(path, datasets, compress, shuffle):
    if compress is None:
        return h5.write(path, datasets)
    chunks = {k: _slabs(np.shape(v)) for k, v in datasets.items() if np.ndim(v) > 0}
    return h5.write(path, datasets, chunks=chunks, deflate=compress, shuffle=shuffle)


# ------------------------------------------------------------------------- grid files


def write_metrics(path: str, m, J, compress: int | None = 3) -> str:
    """metrics.h5 (parse_mesh.jl:250-261): the nine metrics (dxi/dx ... dzeta/dz, cofactors
    scaled by J^-1) and J, each (Nz+8, Ny+8, Nx+8) Float32, deflated at `compress`."""
    if len(m) != 9:
        raise ValueError("nine metric arrays are needed")
    data = {name: _host(a) for name, a in zip(METRIC_NAMES, m)}
    data["J"] = _host(J)
    shapes = {a.shape for a in data.values()}
    if len(shapes) != 1 or len(next(iter(shapes))) != 3:
        raise ValueError("metrics and J must be (Nz+8, Ny+8, Nx+8) arrays of one shape")
    return _write(path, data, compress, False)


def read_metrics(path: str, dtype=np.float64) -> tuple[list, np.ndarray]:
    """([nine metrics], J) from metrics.h5 as `dtype` (solver.jl:237-250 reads the whole
    arrays on one rank)."""
    with h5.H5File(path) as f:
        missing = [k for k in METRIC_NAMES + ("J",) if k not in f]
        if missing:
            raise KeyError(f"{path}: no dataset {missing[0]!r}")
        return [f[k].astype(dtype) for k in METRIC_NAMES], f["J"].astype(dtype)


def write_mesh(path: str, x, y, z, compress: int | None = 3) -> str:
    """mesh.h5 (parse_mesh.jl:262-273): NG, Nx, Ny, Nz as Int64 scalars and the interior
    coordinates as coords (Nz, Ny, Nx, 3) Float32 (Julia (3, Nx, Ny, Nz)); x, y, z are
    (Nz+8, Ny+8, Nx+8) with ghosts, as the grid pipeline makes them."""
    X, Y, Z = (_host(a) for a in (x, y, z))
    if X.ndim != 3 or Y.shape != X.shape or Z.shape != X.shape:
        raise ValueError("x, y, z must be (Nz+8, Ny+8, Nx+8) arrays of one shape")
    nz, ny, nx = (n - 2 * NG for n in X.shape)
    coords = np.stack([_interior(A) for A in (X, Y, Z)], axis=-1)
    data = {"NG": np.int64(NG), "Nx": np.int64(nx), "Ny": np.int64(ny), "Nz": np.int64(nz), "coords": coords}
    return _write(path, data, compress, False)


def read_mesh(path: str, dtype=np.float32) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """x, y, z ((Nz+8, Ny+8, Nx+8) of `dtype`) from mesh.h5: the interior coordinates, then
    the ghost layers by the solver's extrapolation (solver.jl:252-274 on one rank; Float32
    arrays there)."""
    with h5.H5File(path) as f:
        ng, nx, ny, nz = (int(f[k]) for k in ("NG", "Nx", "Ny", "Nz"))
        coords = f["coords"]
    if ng != NG or coords.shape != (nz, ny, nx, 3):
        raise ValueError(f"{path}: NG={ng}, coords {coords.shape} for Nx,Ny,Nz = {nx},{ny},{nz}")
    shape = (nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)
    out = []
    for d in range(3):
        A = np.zeros(shape, dtype=dtype)
        A[NG:-NG, NG:-NG, NG:-NG] = coords[..., d]
        out.append(A)
    return extend_ghosts(*out, dtype=dtype, rule="solver")


# ------------------------------------------------------------------------- solution files


def write_XDMF(plt_dir: str, tt: int, dt: float, nx: int, ny: int, nz: int, mesh: str = "./mesh.h5") -> str:
    """PLT/plt-tt.xmf (IO.jl:236-292): an XDMF 2.2 description of plt-tt.h5 on the
    curvilinear mesh (3DSMesh, XYZ geometry from mesh.h5:/coords), time tt*dt, the seven
    node-centred Float32 scalars rho u v w p T phi."""
    h5name = f"plt-{tt}.h5"
    dims = f"{nz} {ny} {nx}"
    lines = ['<?xml version="1.0" ?>',
             '<!DOCTYPE Xdmf SYSTEM "Xdmf.dtd" []>',
             '<Xdmf xmlns:xi="http://www.w3.org/2003/XInclude" Version="2.2">',
             ' <Domain>',
             '  <Grid Name="Grid" GridType="Uniform">',
             f'  <Time Value="{tt * dt}" />',
             f'   <Topology TopologyType="3DSMesh" NumberOfElements="{dims}" />',
             '   <Geometry GeometryType="XYZ">',
             f'   <DataItem Name="coords" Dimensions="{dims} 3" NumberType="Float" Precision="4" Format="HDF">',
             f'    {mesh}:/coords',
             '   </DataItem>',
             '   </Geometry>']
    for name in PRIM_NAMES + ("phi",):
        lines += [f'   <Attribute Name="{name}" AttributeType="Scalar" Center="Node">',
                  f'    <DataItem Dimensions="{dims}" NumberType="Float" Precision="4" Format="HDF">',
                  f'    {h5name}:/{name}',
                  '   </DataItem>',
                  '   </Attribute>']
    lines += ['  </Grid>', ' </Domain>', '</Xdmf>']
    os.makedirs(plt_dir, exist_ok=True)
    path = os.path.join(plt_dir, f"plt-{tt}.xmf")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def plotFile_xdmf(out_dir: str, tt: int, Q, phi, dt: float, shuffle: bool = True,
                  compress: int | None = 1) -> str:
    """PLT/plt-tt.h5 with the interior rho, u, v, w, p, T and the shock sensor phi as
    separate (Nz, Ny, Nx) Float32 datasets, and its XDMF file (IO.jl:1-112). Q is (6, Nz+8,
    Ny+8, Nx+8), phi (Nz+8, Ny+8, Nx+8)."""
    Qh, ph = _interior(_host(Q)), _interior(_host(phi))
    if Qh.shape[0] != 6 or ph.shape != Qh.shape[1:]:
        raise ValueError("Q must be (6, Nz+8, Ny+8, Nx+8) and phi (Nz+8, Ny+8, Nx+8)")
    plt_dir = os.path.join(out_dir, "PLT")
    os.makedirs(plt_dir, exist_ok=True)
    write_XDMF(plt_dir, tt, dt, Qh.shape[3], Qh.shape[2], Qh.shape[1])
    data = {name: Qh[n] for n, name in enumerate(PRIM_NAMES)}
    data["phi"] = ph
    return _write(os.path.join(plt_dir, f"plt-{tt}.h5"), data, compress, shuffle)


def plotFile_h5(out_dir: str, tt: int, Q, shuffle: bool = True, compress: int | None = 1) -> str:
    """PLT/plt-tt.h5 with one dataset Q: the interior primitives (6, Nz, Ny, Nx) Float32
    (IO.jl:114-151, Julia (Nx, Ny, Nz, 6))."""
    Qh = np.ascontiguousarray(_interior(_host(Q)))
    if Qh.ndim != 4 or Qh.shape[0] != 6:
        raise ValueError("Q must be (6, Nz+8, Ny+8, Nx+8)")
    plt_dir = os.path.join(out_dir, "PLT")
    os.makedirs(plt_dir, exist_ok=True)
    return _write(os.path.join(plt_dir, f"plt-{tt}.h5"), {"Q": Qh}, compress, shuffle)


def checkpointFile(out_dir: str, tt: int, Q, shuffle: bool = True, compress: int | None = 1) -> str:
    """CHK/chk-tt.h5 with Q_h: the primitives with ghosts, (ranks=1, 6, Nz+8, Ny+8, Nx+8)
    Float32 (IO.jl:153-183)."""
    Qh = _host(Q)
    if Qh.ndim != 4 or Qh.shape[0] != 6:
        raise ValueError("Q must be (6, Nz+8, Ny+8, Nx+8)")
    chk_dir = os.path.join(out_dir, "CHK")
    os.makedirs(chk_dir, exist_ok=True)
    Qr = Qh[None]
    return _write(os.path.join(chk_dir, f"chk-{tt}.h5"), {"Q_h": Qr}, compress, shuffle)


def read_checkpoint(path: str, rank: int = 0, dtype=np.float32) -> np.ndarray:
    """Q (6, Nz+8, Ny+8, Nx+8) of `rank` from a checkpoint's Q_h (solver.jl:211-216 takes
    Q_h[..., :, 1] on one rank)."""
    with h5.H5File(path) as f:
        Qh = f["Q_h"]
    if Qh.ndim != 5 or Qh.shape[1] != 6 or not 0 <= rank < Qh.shape[0]:
        raise ValueError(f"{path}: Q_h of shape {Qh.shape}, rank {rank}")
    return Qh[rank].astype(dtype)


def assemble_checkpoint(path: str, nprocs=(1, 1, 1), dtype=np.float32) -> np.ndarray:
    """The global Q (6, Nz+8, Ny+8, Nx+8) from the checkpoint of a run on px x py x pz ranks,
    to restart it on one GPU. Each rank wrote its local block with its ghost frame
    (IO.jl:153-183, Q_h[..., rank+1]); ranks are numbered as MPI_Cart_create numbers them
    (run.jl:117: row-major, z fastest). Every block lands at its rank's offset, then every
    block's interior over the halos, so the global ghost frame comes from the blocks on the
    domain faces. (The reference's own restart, solver.jl:211-216, reads one rank.)"""
    with h5.H5File(path) as f:
        Qh = f["Q_h"]
    px, py, pz = nprocs
    if Qh.ndim != 5 or Qh.shape[0] != px * py * pz or Qh.shape[1] != 6:
        raise ValueError(f"{path}: Q_h of shape {Qh.shape} for {px}x{py}x{pz} ranks")
    nzp, nyp, nxp = (n - 2 * NG for n in Qh.shape[2:])
    G = np.zeros((6, pz * nzp + 2 * NG, py * nyp + 2 * NG, px * nxp + 2 * NG), dtype)

    def at(r, inner):
        cx, cy, cz = r // (py * pz), (r // pz) % py, r % pz
        o = 0 if not inner else NG
        return (slice(None), slice(cz * nzp + o, (cz + 1) * nzp + 2 * NG - o),
                slice(cy * nyp + o, (cy + 1) * nyp + 2 * NG - o), slice(cx * nxp + o, (cx + 1) * nxp + 2 * NG - o))

    for r in range(Qh.shape[0]):
        G[at(r, False)] = Qh[r]
    for r in range(Qh.shape[0]):
        G[at(r, True)] = _interior(Qh[r])
    return G


def averageFile(out_dir: str, tt: int, Q_avg, shuffle: bool = True, compress: int | None = 1) -> str:
    """AVG/avg-tt.h5 with avg: the interior of the averaged primitives (6, Nz, Ny, Nx)
    Float32 (IO.jl:185-210)."""
    A = np.ascontiguousarray(_interior(_host(Q_avg)))
    if A.ndim != 4 or A.shape[0] != 6:
        raise ValueError("Q_avg must be (6, Nz+8, Ny+8, Nx+8)")
    avg_dir = os.path.join(out_dir, "AVG")
    os.makedirs(avg_dir, exist_ok=True)
    return _write(os.path.join(avg_dir, f"avg-{tt}.h5"), {"avg": A}, compress, shuffle)
