"""The reference's grid generators and its CPU metrics, restated (host-side set-up code).

  swept_ramp_mesh   SCU-benchmark/swept-compression-ramp.c:180-449 (and its output files,
                    write_swept_outputs, :446-560): the swept compression
                    ramp written to OCFD3d-Mesh.dat (Hermite-stretched inlet, the corner arc
                    of the upper boundary, exponential wall-normal stretching whose exponent
                    Newton's method finds, wall orthogonalisation, spanwise sweep), for the
                    single process or the z slabs of N processes;
  flat_plate_grid   parse_mesh.jl:20-136: the flat plate with sinh wall-normal stretching in
                    Float32, ghosts by point reflection (the solver's extrapolation rule);
  metrics_f32       the Float32 metrics and J that fill metrics.h5: readfort.jl:103-209
                    (Float32 difference coefficients) or parse_mesh.jl:138-248 (Float64
                    coefficients on Float32 differences, rounded to Float32);
  reference_files   metrics.h5 and mesh.h5 from either pipeline (readfort.jl: OCFD mesh in
                    millimetres, Float32, ghosts, metres; parse_mesh.jl: the flat plate).

The arithmetic follows the reference's operation order. Julia and C (compiled without
multiply-add contraction, as on x86-64 by default) round every operation, as numpy does, so
the Float32 metrics and the ramp coordinates are those of the reference's own programs; the
transcendental functions come from this platform's libm (math module), as the C program's.

  python -m flame3d_mhd_gb300.meshgen swept --params swept-compression-grid.in --out DIR [--metrics]
  python -m flame3d_mhd_gb300.meshgen plate --out DIR
"""
from __future__ import annotations

import argparse
import math
import os
import sys

import numpy as np

from . import files, vtk
from .grid import NG, extend_ghosts, mesh_from_ocfd, write_ocfd_mesh

PI = 3.1415926535897932  # swept-compression-ramp.c:8

# swept-compression-grid.in of the reference (SCU-benchmark)
SWEPT_DEFAULTS = dict(nx=1000, ny=240, nz=100, nprocs=1, nx_inlet=680, nx_corner=300, nx_buff=20,
                      dx_inlet=0.5, lx_inlet=300.0, lx_corner=50.0, alfax_buff=1.05, sw_angle=0.0,
                      comp_angle=24.0, high=35.0, hy_wall=0.01, lz=14.0)
_SWEPT_FIELDS = (("nx", "ny", "nz", "nprocs"), ("nx_inlet", "nx_corner", "nx_buff"),
                 ("dx_inlet", "lx_inlet", "lx_corner", "alfax_buff"), ("sw_angle", "comp_angle"),
                 ("high", "hy_wall", "lz"), ("tec1", "mesh2d", "tec2"))


def read_swept_params(path: str) -> dict:
    """The parameter file of swept-compression-ramp.c (Read_parameter, :78-105): six
    pairs of a title line and a line of values."""
    lines = [ln for ln in open(path).read().splitlines()]
    out = {}
    for n, names in enumerate(_SWEPT_FIELDS):
        vals = lines[2 * n + 1].split()
        if len(vals) < len(names):
            raise ValueError(f"{path}: line {2 * n + 2} needs {len(names)} values")
        for name, v in zip(names, vals):
            out[name] = int(v) if name in ("nx", "ny", "nz", "nprocs", "nx_inlet", "nx_corner", "nx_buff",
                                           "tec1", "mesh2d", "tec2") else float(v)
    return out


def _pow2(v: np.ndarray, square: str = "libm") -> np.ndarray:
    """pow(v, 2) as the C program squares: libm's pow per element (square="libm", the program
    built without optimisation or with -fno-builtin), or v*v (square="mul": gcc -O1 and above
    replace pow(v, 2.0) by a multiplication). glibc's pow is within 0.52 ulp, not correctly
    rounded, so the two can differ in the last bit."""
    if square == "mul":
        return v * v
    return np.array([math.pow(t, 2.0) for t in v.tolist()])


def _inlet_x(n: int, length: float, dx1: float, dx2: float) -> list:
    """gridx_inlet (:180-197): n points on [0, length], cubic Hermite in the index with end
    spacings dx1 and dx2."""
    out = []
    for i in range(1, n + 1):
        x = (i - 1.0) / (n - 1.0)
        ah1 = (1.0 - 2.0 * (x - 1.0)) * x * x
        sh0 = x * (x - 1.0) ** 2
        sh1 = (x - 1.0) * x * x
        out.append(length * ah1 + dx1 * (n - 1.0) * sh0 + dx2 * (n - 1.0) * sh1)
    return out


def swept_ramp_mesh(p: dict | None = None, with_2d: bool = False, square: str = "libm", **kw) -> tuple:
    """Coordinates (Nz, Ny, Nx) float64 of swept-compression-ramp.c for the parameters `p`
    (SWEPT_DEFAULTS, updated by keyword arguments): the lower wall xa, ya and the upper
    boundary xb, yb along xi (gridx, :199-236), points between them on an exponential
    distribution whose first spacing is hy_wall (gridxy, :238-275), the first 19 grid lines
    off the wall made orthogonal to it (Wall_Orthonormalization, :385-426), then the spanwise
    extrusion with the inlet stretched by the sweep (gridxyz, :277-383), for the z slab of
    each of `nprocs` processes. with_2d: also the (Ny, Nx) plane x, y it extrudes. square: how
    the orthogonalisation squares (_pow2): "libm" reproduces the program built at gcc's default
    optimisation level, "mul" the program built with -O2."""
    if square not in ("libm", "mul"):
        raise ValueError("square must be 'libm' or 'mul'")
    q = dict(SWEPT_DEFAULTS)
    q.update(p or {})
    q.update(kw)
    nx, ny, nz, nproc = q["nx"], q["ny"], q["nz"], q["nprocs"]
    ni, nc, nb = q["nx_inlet"], q["nx_corner"], q["nx_buff"]
    if ni + nc + nb != nx:
        raise ValueError("nx_inlet + nx_corner + nx_buff != nx")
    if ny < 20:
        raise ValueError("ny < 20: the wall orthogonalisation moves grid lines 1-19")
    if nc < 2 or ni < 2:
        raise ValueError("nx_inlet and nx_corner need two points or more")
    Li, Lc, alfa = q["lx_inlet"], q["lx_corner"], q["alfax_buff"]
    high, hy_wall, Lz = q["high"], q["hy_wall"], q["lz"]
    sw = q["sw_angle"] * PI / 180.0
    comp = q["comp_angle"] * PI / 180.0
    hx0 = 2.0 * Lc / (nc - 1)
    R = Lc / math.tan(comp / 2.0) - high

    # gridx: the lower wall (a) and the upper boundary (b)
    xa, ya, xb, yb = [0.0] * nx, [0.0] * nx, [0.0] * nx, [0.0] * nx
    xa[:ni] = _inlet_x(ni + 1, Li, q["dx_inlet"], hx0)[:ni]
    for i in range(ni):
        xa[i] = xa[i] - Lc - Li
        ya[i] = 0.0
        xb[i] = xa[i]
        yb[i] = high
    for i in range(nc):
        seta = comp * i / (nc - 1.0)
        if seta < comp / 2:
            xa[i + ni] = i * hx0 - Lc
            ya[i + ni] = 0.0
        else:
            xa[i + ni] = (i * hx0 - Lc) * math.cos(comp)
            ya[i + ni] = (i * hx0 - Lc) * math.sin(comp)
        xb[i + ni] = R * math.sin(seta) - Lc
        yb[i + ni] = R * (1.0 - math.cos(seta)) + high
    t = math.tan(comp)
    for i in range(nb):
        n = i + ni + nc
        dx = (xa[n - 1] - xa[n - 2]) * alfa
        xa[n] = xa[n - 1] + dx
        ya[n] = ya[n - 1] + dx * t
        xb[n] = xb[n - 1] + dx
        yb[n] = yb[n - 1] + dx * t

    # gridxy: the stretching exponent b of (exp(b s) - 1) / (exp(b) - 1) from Newton's
    # method, started at 3.5; the reference's loop counter is not reset between columns, so
    # the first column takes ten Newton steps and every later one a single step from the
    # previous column's b (:246-259)
    x2 = np.zeros((ny, nx))
    y2 = np.zeros((ny, nx))
    b, count = 3.5, 0
    m = ny - 1.0
    for i in range(nx):
        SL = math.sqrt((xb[i] - xa[i]) ** 2 + (yb[i] - ya[i]) ** 2)
        dy = 1.0 / (ny - 1.0)
        delta = hy_wall / SL
        while True:
            e1, eb = math.exp(b / m), math.exp(b)
            fb = (e1 - 1.0) / (eb - 1.0) - delta
            fbx = (e1 / m * (eb - 1.0) - (e1 - 1.0) * eb) / (eb - 1.0) ** 2
            b = b - fb / fbx
            count += 1
            if count >= 10:
                break
        a = 1.0 / (math.exp(b) - 1.0)
        for j in range(ny):
            sy = a * (math.exp(j * dy * b) - 1)
            x2[j, i] = xa[i] + (xb[i] - xa[i]) * sy
            y2[j, i] = ya[i] + (yb[i] - ya[i]) * sy

    # Wall_Orthonormalization: ten sweeps over grid lines 1-19; each interior point moves
    # toward the foot of the normal from the line below, by a 1-2-1 smoothed correction
    # weighted exp(-3 j / 20) / 2 (elementwise IEEE operations, vectorised along xi)
    for _ in range(10):
        for j in range(1, 20):
            ex, ey = x2[j, 2:] - x2[j, :-2], y2[j, 2:] - y2[j, :-2]
            qn = np.sqrt(_pow2(ex, square) + _pow2(ey, square))
            qnx, qny = -ey / qn, ex / qn
            rx, ry = x2[j, 1:-1] - x2[j - 1, 1:-1], y2[j, 1:-1] - y2[j - 1, 1:-1]
            s = rx * qnx + ry * qny
            dxv = np.zeros(nx)
            dyv = np.zeros(nx)
            dxv[1:-1] = s * qnx - rx
            dyv[1:-1] = s * qny - ry
            w = math.exp(-3.0 * j / 20) / 2.0
            x2[j, 1:-1] = x2[j, 1:-1] + w * ((dxv[:-2] + 2.0 * dxv[1:-1] + dxv[2:]) / 4.0)
            y2[j, 1:-1] = y2[j, 1:-1] + w * ((dyv[:-2] + 2.0 * dyv[1:-1] + dyv[2:]) / 4.0)

    # gridxyz: the z slabs of the processes (the first nz % N hold one plane more)
    x3 = np.empty((nz, ny, nx))
    y3 = np.empty((nz, ny, nx))
    z3 = np.empty((nz, ny, nx))
    npz = [nz // nproc + (1 if r < nz % nproc else 0) for r in range(nproc)]
    np0 = [sum(npz[:r]) for r in range(nproc)]
    ts = math.tan(sw)
    for r in range(nproc):
        NZ = npz[r]
        if NZ < 2:
            raise ValueError(f"process {r} holds {NZ} plane(s): the reference's z formula divides by zero")
        for k in range(NZ):
            z = k * Lz * (npz[r] - 1) / ((NZ - 1) * (nz - 1)) + np0[r] * Lz / (nz - 1)
            F = Li - Lz * ts + Lz / (nz - 1) * (k + np0[r]) * ts
            kk = np0[r] + k
            x3[kk, :, :ni] = (x2[:, :ni] - x2[:, :1]) * F / Li + x2[:, :1]
            x3[kk, :, ni:] = x3[kk, :, ni - 1:ni] + x2[:, ni:] - x2[:, ni - 1:ni]
            y3[kk] = y2
            z3[kk] = z
    return (x3, y3, z3, x2, y2) if with_2d else (x3, y3, z3)


def write_swept_outputs(out_dir: str, p: dict, x3, y3, z3, x2, y2) -> list:
    """The files of swept-compression-ramp.c's output() (:446-560): OCFD3d-Mesh.dat; y1d.dat
    (the first column's y, "%15.6f"); with Tec1 gridxy.dat and with Tec2 grid.dat (Tecplot
    text of the plane and of the grid); with Mesh2D OCFD2d-Mesh.dat (x and y of the plane,
    each one record). Returns the paths written."""
    os.makedirs(out_dir, exist_ok=True)
    nz, ny, nx = x3.shape
    out = [os.path.join(out_dir, "OCFD3d-Mesh.dat")]
    write_ocfd_mesh(out[0], x3, y3, z3)
    path = os.path.join(out_dir, "y1d.dat")
    with open(path, "w") as f:
        f.writelines(f"{v:15.6f}\n" for v in y2[:, 0].tolist())
    out.append(path)
    if p.get("tec1", 1) == 1:
        path = os.path.join(out_dir, "gridxy.dat")
        with open(path, "w") as f:
            f.write(f"variables=x,y\nzone i={nx} ,j={ny}\n")
            f.writelines(f"{a:15.6f}{b:15.6f}\n" for a, b in zip(x2.ravel().tolist(), y2.ravel().tolist()))
        out.append(path)
    if p.get("mesh2d", 1) == 1:
        path = os.path.join(out_dir, "OCFD2d-Mesh.dat")
        mark = np.array([nx * ny * 8], dtype="<i4").tobytes()
        with open(path, "wb") as f:
            for a in (x2, y2):
                f.write(mark + np.ascontiguousarray(a, dtype="<f8").tobytes() + mark)
        out.append(path)
    if p.get("tec2", 0) == 1:
        path = os.path.join(out_dir, "grid.dat")
        with open(path, "w") as f:
            f.write(f"variables=x,y,z\nzone i={nx} ,j={ny} ,k={nz}\n")
            for k in range(nz):
                f.writelines(f"{a:15.6f}{b:15.6f}{c:15.6f}\n" for a, b, c in
                             zip(x3[k].ravel().tolist(), y3[k].ravel().tolist(), z3[k].ravel().tolist()))
        out.append(path)
    return out


def flat_plate_grid(nx: int = 256, ny: int = 128, nz: int = 32, lx: float = 2.0, ly: float = 0.1,
                    lz: float = 0.1, factor: float = 3.5) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """parse_mesh.jl's flat plate (:20-136): (Nz+8, Ny+8, Nx+8) Float32 coordinates,
    x = Lx xi, y = Ly sinh(f eta) / sinh(f), z = Lz zeta on the unit computational cube,
    every ghost layer then set by point reflection (the solver's extrapolation rule, which
    parse_mesh.jl:75-136 applies). sinh is the correctly rounded Float32 value; Julia's own
    Float32 sinh may differ in the last bit."""
    f32 = np.float32
    shape = (nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)
    xi = (np.arange(nx, dtype=f32) / f32(nx - 1))
    eta = (np.arange(ny, dtype=f32) / f32(ny - 1))
    zeta = (np.arange(nz, dtype=f32) / f32(nz - 1))
    fac, Ly = f32(factor), f32(ly)
    sh = lambda v: np.sinh(np.asarray(v, np.float64)).astype(f32)
    yv = (Ly * sh(fac * eta)) / sh(fac)
    X, Y, Z = (np.zeros(shape, f32) for _ in range(3))
    I = (slice(NG, -NG),) * 3
    X[I] = (f32(lx) * xi)[None, None, :]
    Y[I] = yv[None, :, None]
    Z[I] = (f32(lz) * zeta)[:, None, None]
    return extend_ghosts(X, Y, Z, dtype=f32, rule="solver")


def metrics_f32(x, y, z, coefficients: str = "readfort") -> tuple[list, np.ndarray]:
    """The Float32 metrics and J of the reference's CPU set-up ((Nz+8, Ny+8, Nx+8) each, the
    nine metrics in metrics.h5 order): sixth-order central differences inside, second-order
    one-sided ones in the three outer layers of each direction, J = 1 / det, the cofactors
    (readfort.jl:103-181, parse_mesh.jl:138-248). coefficients="readfort": Float32
    coefficients (1/60f0 ...); "parse_mesh": Float64 coefficients applied to Float32
    differences, rounded to Float32 when stored."""
    if coefficients not in ("readfort", "parse_mesh"):
        raise ValueError("coefficients: 'readfort' or 'parse_mesh'")
    f32, f64 = np.float32, np.float64
    X, Y, Z = (np.asarray(a, f32) for a in (x, y, z))

    def d(f, axis):
        f = np.moveaxis(f, axis, -1)
        n = f.shape[-1]
        out = np.empty_like(f)
        s = lambda a, b: f[..., a:n - b] if b else f[..., a:]
        d1, d2, d3 = s(4, 2) - s(2, 4), s(5, 1) - s(1, 5), s(6, 0) - s(0, 6)  # f[i+1]-f[i-1], ...
        if coefficients == "readfort":
            out[..., 3:n - 3] = f32(1) / f32(60) * d3 - f32(3) / f32(20) * d2 + f32(3) / f32(4) * d1
            out[..., :3] = f32(2) * f[..., 1:4] - f32(0.5) * f[..., 2:5] - f32(1.5) * f[..., 0:3]
            out[..., n - 3:] = f32(-2) * f[..., n - 4:n - 1] + f32(0.5) * f[..., n - 5:n - 2] + f32(1.5) * f[..., n - 3:]
        else:
            out[..., 3:n - 3] = ((1 / 60) * d3.astype(f64) - (3 / 20) * d2.astype(f64)
                                 + (3 / 4) * d1.astype(f64)).astype(f32)
            out[..., :3] = ((f32(2) * f[..., 1:4]).astype(f64) - 0.5 * f[..., 2:5].astype(f64)
                            - 1.5 * f[..., 0:3].astype(f64)).astype(f32)
            out[..., n - 3:] = ((f32(-2) * f[..., n - 4:n - 1]).astype(f64) + 0.5 * f[..., n - 5:n - 2].astype(f64)
                                + 1.5 * f[..., n - 3:].astype(f64)).astype(f32)
        return np.moveaxis(out, -1, axis)

    xxi, yxi, zxi = d(X, 2), d(Y, 2), d(Z, 2)
    xet, yet, zet = d(X, 1), d(Y, 1), d(Z, 1)
    xze, yze, zze = d(X, 0), d(Y, 0), d(Z, 0)
    J = f32(1) / (xxi * (yet * zze - yze * zet) - xet * (yxi * zze - yze * zxi) + xze * (yxi * zet - yet * zxi))
    m = [yet * zze - yze * zet, xze * zet - xet * zze, xet * yze - xze * yet,
         yze * zxi - yxi * zze, xxi * zze - xze * zxi, xze * yxi - xxi * yze,
         yxi * zet - yet * zxi, xet * zxi - xxi * zet, xxi * yet - xet * yxi]
    return m, J


def reference_files(out_dir: str, x, y, z, coefficients: str = "readfort", vis: bool = False) -> tuple:
    """metrics.h5 and mesh.h5 as the reference's set-up writes them from ghost-filled Float32
    coordinates: readfort.jl (deflate level 0, stored uncompressed here) or parse_mesh.jl
    (deflate level 3); with `vis` also its mesh.vts (J, and the metrics for parse_mesh.jl)."""
    m, J = metrics_f32(x, y, z, coefficients)
    level = None if coefficients == "readfort" else 3
    os.makedirs(out_dir, exist_ok=True)
    out = (files.write_metrics(os.path.join(out_dir, "metrics.h5"), m, J, compress=level),
           files.write_mesh(os.path.join(out_dir, "mesh.h5"), x, y, z, compress=level))
    if vis:
        out += (vtk.write_mesh_vts(os.path.join(out_dir, "mesh.vts"), x, y, z, J,
                                   m if coefficients == "parse_mesh" else None),)
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    s = sub.add_parser("swept", help="swept-compression-ramp.c: OCFD3d-Mesh.dat [and the readfort.jl files]")
    s.add_argument("--params", default="", help="swept-compression-grid.in (default: the reference's values)")
    s.add_argument("--out", default=".")
    s.add_argument("--metrics", action="store_true", help="also metrics.h5 and mesh.h5 as readfort.jl makes them")
    s.add_argument("--vis", action="store_true", help="and mesh.vts (readfort.jl's vis)")
    p = sub.add_parser("plate", help="parse_mesh.jl: the flat plate's metrics.h5 and mesh.h5")
    p.add_argument("--nx", type=int, default=256)
    p.add_argument("--ny", type=int, default=128)
    p.add_argument("--nz", type=int, default=32)
    p.add_argument("--out", default=".")
    p.add_argument("--vis", action="store_true", help="also mesh.vts (parse_mesh.jl's vis)")
    a = ap.parse_args(argv)
    os.makedirs(a.out, exist_ok=True)
    if a.cmd == "swept":
        q = read_swept_params(a.params) if a.params else dict(SWEPT_DEFAULTS, tec1=1, mesh2d=1, tec2=0)
        paths = write_swept_outputs(a.out, q, *swept_ramp_mesh(q, with_2d=True))
        print(*paths)
        path = paths[0]
        if a.metrics:
            X, Y, Z = mesh_from_ocfd(path, q["nx"], q["ny"], q["nz"])
            print(*reference_files(a.out, X, Y, Z, "readfort", vis=a.vis))
    else:
        X, Y, Z = flat_plate_grid(a.nx, a.ny, a.nz)
        print(*reference_files(a.out, X, Y, Z, "parse_mesh", vis=a.vis))
    return 0


if __name__ == "__main__":
    sys.exit(main())
