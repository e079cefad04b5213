"""Grid pipeline: ghost-cell coordinates and analytic body-fitted grids.

Host-side set-up code (it runs once per grid, before the metrics are computed on the device
by f3d_compute_metrics). Arrays are (Nz+8, Ny+8, Nx+8), the reference's Julia (Nx,Ny,Nz)
column-major arrays seen from C order.
"""
from __future__ import annotations

import numpy as np

NG = 4


def extend_ghosts(x: np.ndarray, y: np.ndarray, z: np.ndarray, dtype=np.float64,
                  rule: str = "readfort") -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Fill the ghost layers of interior coordinates as SCU-benchmark/readfort.jl:34-95 does
    (rule="readfort", the grid pipeline), or as the solver's `extrapolation` does after
    reading mesh.h5 (rule="solver", solver.jl:682-826, one rank).

    Point reflection about the first / last interior cell (x_g = 2 x_b - x_mirror) on the
    xi and eta faces for all three coordinates, except that readfort.jl copies z unreflected
    across the eta faces (readfort.jl:48-58; solver.jl:731-751 reflects it too);
    parallelogram completion x = x[i, b] + x[b, j] - x[b, b] in the four xi-eta edge regions
    (readfort.jl:61-83, solver.jl:753-795); then point reflection on the zeta faces over the
    full xi-eta extent (readfort.jl:85-95, solver.jl:797-823). Interior values are untouched.
    Returns new arrays of `dtype` (arithmetic in that type: np.float32 repeats the Float32
    arrays of the reference); inputs are (Nz+8, Ny+8, Nx+8) with the interior filled.
    """
    if rule not in ("readfort", "solver"):
        raise ValueError(f"rule {rule!r}: 'readfort' or 'solver'")
    X, Y, Z = (np.array(a, dtype=dtype, copy=True) for a in (x, y, z))
    nzt, nyt, nxt = X.shape
    nx, ny = nxt - 2 * NG, nyt - 2 * NG
    ki = slice(NG, nzt - NG)  # interior k
    ji = slice(NG, nyt - NG)
    ii = slice(NG, nxt - NG)
    lo_i, hi_i = NG, NG + nx - 1  # first / last interior (0-based)
    lo_j, hi_j = NG, NG + ny - 1
    for A in (X, Y, Z):
        # xi faces (readfort.jl:34-46): A[g] = 2 A[b] - A[2b - g]
        for g in range(NG):
            A[ki, ji, g] = 2 * A[ki, ji, lo_i] - A[ki, ji, 2 * lo_i - g]
            gh = hi_i + 1 + g
            A[ki, ji, gh] = 2 * A[ki, ji, hi_i] - A[ki, ji, 2 * hi_i - gh]
    for A, reflect in ((X, True), (Y, True), (Z, rule == "solver")):
        # eta faces (readfort.jl:48-58: z is copied from the mirror cell)
        for g in range(NG):
            gh = hi_j + 1 + g
            if reflect:
                A[ki, g, ii] = 2 * A[ki, lo_j, ii] - A[ki, 2 * lo_j - g, ii]
                A[ki, gh, ii] = 2 * A[ki, hi_j, ii] - A[ki, 2 * hi_j - gh, ii]
            else:
                A[ki, g, ii] = A[ki, 2 * lo_j - g, ii]
                A[ki, gh, ii] = A[ki, 2 * hi_j - gh, ii]
    for A in (X, Y, Z):
        # xi-eta edges (readfort.jl:61-83)
        jl, jh = slice(0, NG), slice(hi_j + 1, nyt)
        il, ih = slice(0, NG), slice(hi_i + 1, nxt)
        for js, jb in ((jl, lo_j), (jh, hi_j)):
            for is_, ib in ((il, lo_i), (ih, hi_i)):
                A[ki, js, is_] = (A[ki, jb, is_][:, None, :] + A[ki, js, ib][:, :, None]
                                  - A[ki, jb, ib][:, None, None])
        # zeta faces over the full xi-eta extent (readfort.jl:85-95)
        lo_k, hi_k = NG, nzt - NG - 1
        for g in range(NG):
            A[g] = 2 * A[lo_k] - A[2 * lo_k - g]
            gh = hi_k + 1 + g
            A[gh] = 2 * A[hi_k] - A[2 * hi_k - gh]
    return X, Y, Z


def tanh_beta(n: int, height: float, first: float) -> float:
    """Stretching parameter of s(eta) = 1 - tanh(beta (1 - eta)) / tanh(beta) for which the
    first of n cells spanning `height` is `first` high (bisection; s(1/n) decreases in beta)."""
    target = first / height
    if not 0.0 < target < 1.0 / n:
        raise ValueError("first cell must be smaller than the uniform spacing")
    s1 = lambda b: 1.0 - np.tanh(b * (1.0 - 1.0 / n)) / np.tanh(b)
    lo, hi = 1e-6, 50.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if s1(mid) > target:
            lo = mid
        else:
            hi = mid
    return 0.5 * (lo + hi)


def ramp_wall(x: np.ndarray, angle_deg: float, corner_radius: float) -> np.ndarray:
    """Wall height of a compression ramp with its corner at x = 0: 0 upstream, rising at
    `angle_deg` downstream, the corner rounded over ~corner_radius (softplus blend)."""
    t = np.tan(np.radians(angle_deg))
    return t * corner_radius * np.logaddexp(0.0, x / corner_radius)


def compression_ramp_grid(nx: int, ny: int, nz: int, angle_deg: float = 24.0, x_up: float = 8.0,
                          x_down: float = 8.0, height: float = 10.0, span: float = 4.0,
                          first_cell: float = 1e-3, corner_radius: float = 0.5):
    """Cell-centred body-fitted grid of a compression ramp (lengths in inflow boundary-layer
    thicknesses): uniform in x on [-x_up, x_down] and in z on [0, span); wall-normal lines
    vertical, y = y_w(x) + (height - y_w(x)) s(eta) with tanh stretching whose first cell at
    the inflow is `first_cell` high; the wall is the eta = 0 face. Ghost coordinates as the
    reference's grid pipeline extends them (extend_ghosts)."""
    nxt, nyt, nzt = nx + 2 * NG, ny + 2 * NG, nz + 2 * NG
    beta = tanh_beta(ny, height, first_cell)
    xs = -x_up + (np.arange(nx) + 0.5) * (x_up + x_down) / nx
    eta = (np.arange(ny) + 0.5) / ny
    zs = (np.arange(nz) + 0.5) * span / nz
    s = 1.0 - np.tanh(beta * (1.0 - eta)) / np.tanh(beta)
    yw = ramp_wall(xs, angle_deg, corner_radius)
    x = np.zeros((nzt, nyt, nxt))
    y = np.zeros_like(x)
    z = np.zeros_like(x)
    I = (slice(NG, NG + nz), slice(NG, NG + ny), slice(NG, NG + nx))
    x[I] = xs[None, None, :]
    y[I] = (yw[None, :] + (height - yw[None, :]) * s[:, None])[None, :, :]
    z[I] = zs[:, None, None]
    x, y, z = extend_ghosts(x, y, z)
    return x, y, z, beta


# ---- the mesh file of the reference's grid generator -----------------------------------
# SCU-benchmark/swept-compression-ramp.c:451-560 writes OCFD3d-Mesh.dat as Fortran
# unformatted sequential records: for x, then y, then z, one record per zeta plane k, each
# a 4-byte length nx*ny*8, the nx*ny doubles of the plane (xi fastest) and the length again.
# readfort.jl:14-33 reads it plane by plane into Float32 arrays.

def write_ocfd_mesh(path: str, x: np.ndarray, y: np.ndarray, z: np.ndarray) -> None:
    """Write interior coordinates ((Nz, Ny, Nx) each) in the OCFD3d-Mesh.dat record layout."""
    shape = x.shape
    if y.shape != shape or z.shape != shape or len(shape) != 3:
        raise ValueError("x, y, z must be (Nz, Ny, Nx) arrays of one shape")
    nz, ny, nx = shape
    mark = np.array([nx * ny * 8], dtype="<i4").tobytes()
    with open(path, "wb") as f:
        for a in (x, y, z):
            a = np.ascontiguousarray(a, dtype="<f8")
            for k in range(nz):
                f.write(mark)
                f.write(a[k].tobytes())
                f.write(mark)


def read_ocfd_mesh(path: str, nx: int, ny: int, nz: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Interior coordinates ((Nz, Ny, Nx) float64 each) from an OCFD3d-Mesh.dat file; every
    record length is checked (a file of other dimensions or a damaged file raises)."""
    rec = nx * ny * 8
    want = 3 * nz * (rec + 8)
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size != want:
        raise ValueError(f"{path}: {raw.size} bytes, expected {want} for {nx}x{ny}x{nz}")
    recs = raw.reshape(3, nz, rec + 8)
    heads = recs[:, :, :4].copy().view("<i4").reshape(3, nz)
    tails = recs[:, :, rec + 4:].copy().view("<i4").reshape(3, nz)
    if not ((heads == rec).all() and (tails == rec).all()):
        raise ValueError(f"{path}: record markers do not match {nx}x{ny} planes")
    data = recs[:, :, 4:rec + 4].copy().view("<f8").reshape(3, nz, ny, nx).astype(np.float64)
    return data[0], data[1], data[2]


def mesh_from_ocfd(path: str, nx: int, ny: int, nz: int, divisor: float = 1000.0,
                   dtype=np.float32) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """readfort.jl's generateXYZ (:14-100): the mesh file's planes into (Nz+8, Ny+8, Nx+8)
    arrays of `dtype` (Float32 there), the ghost layers by extend_ghosts, then every
    coordinate divided by `divisor` in that type (./= 1000.f0 there: millimetres to metres).
    Pass dtype=np.float64 to keep the file's FP64 coordinates for f3d_compute_metrics."""
    xi, yi, zi = read_ocfd_mesh(path, nx, ny, nz)
    shape = (nz + 2 * NG, ny + 2 * NG, nx + 2 * NG)
    I = (slice(NG, NG + nz), slice(NG, NG + ny), slice(NG, NG + nx))
    out = []
    for a in (xi, yi, zi):
        A = np.zeros(shape, dtype=dtype)
        A[I] = a.astype(dtype)
        out.append(A)
    X, Y, Z = extend_ghosts(*out, dtype=dtype)
    d = np.dtype(dtype).type(divisor)
    return X / d, Y / d, Z / d
