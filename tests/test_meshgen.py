"""The reference's grid generators and CPU metrics (CPU): the vectorised restatements
against literal loop restatements of swept-compression-ramp.c and of the Julia metric loops
(bitwise), the generators' geometry, the Float32 metrics against the oracle's FP64 ones, and
the files of both pipelines."""
import math
import os

import numpy as np
import pytest

from flame3d_mhd_gb300 import files, h5, meshgen
from flame3d_mhd_gb300.grid import NG, extend_ghosts, mesh_from_ocfd, read_ocfd_mesh

SMALL = dict(nx=64, ny=24, nz=6, nprocs=1, nx_inlet=40, nx_corner=20, nx_buff=4, dx_inlet=0.9, lx_inlet=30.0,
             lx_corner=8.0, alfax_buff=1.05, sw_angle=0.0, comp_angle=24.0, high=6.0, hy_wall=0.01, lz=3.0)


def _c_program(q):
    """swept-compression-ramp.c (:180-383) statement by statement, scalar, 0-based arrays."""
    nx, ny, nz, N = q["nx"], q["ny"], q["nz"], q["nprocs"]
    ni, nc, nb = q["nx_inlet"], q["nx_corner"], q["nx_buff"]
    PI = 3.1415926535897932
    sw = q["sw_angle"] * PI / 180.
    comp = q["comp_angle"] * PI / 180.
    Lc, Li, High, Lz = q["lx_corner"], q["lx_inlet"], q["high"], q["lz"]
    hx0 = 2. * Lc / (nc - 1)
    R = Lc / math.tan(comp / 2.) - High
    xa, ya, xb, yb = [0.] * nx, [0.] * nx, [0.] * nx, [0.] * nx
    n = ni + 1  # gridx_inlet(nx_inlet + 1, Lx_inlet, dx_inlet, hx0, xa)
    for i in range(1, n + 1):
        x = (i - 1.) / (n - 1.)
        Ah1 = (1. - 2. * (x - 1.)) * x * x
        Sh0 = x * math.pow(x - 1., 2)
        Sh1 = (x - 1.) * x * x
        if i - 1 < nx:
            xa[i - 1] = Li * Ah1 + q["dx_inlet"] * (n - 1.) * Sh0 + hx0 * (n - 1.) * Sh1
    for i in range(ni):
        xa[i] = xa[i] - Lc - Li
        ya[i] = 0.
        xb[i] = xa[i]
        yb[i] = High
    for i in range(nc):
        seta = comp * i / (nc - 1.)
        if seta < comp / 2:
            xa[i + ni] = i * hx0 - Lc
            ya[i + ni] = 0.
        else:
            xa[i + ni] = (i * hx0 - Lc) * math.cos(comp)
            ya[i + ni] = (i * hx0 - Lc) * math.sin(comp)
        xb[i + ni] = R * math.sin(seta) - Lc
        yb[i + ni] = R * (1. - math.cos(seta)) + High
    for i in range(nb):
        dx = (xa[i + ni + nc - 1] - xa[i + ni + nc - 2]) * q["alfax_buff"]
        xa[i + ni + nc] = xa[i + ni + nc - 1] + dx
        ya[i + ni + nc] = ya[i + ni + nc - 1] + dx * math.tan(comp)
        xb[i + ni + nc] = xb[i + ni + nc - 1] + dx
        yb[i + ni + nc] = yb[i + ni + nc - 1] + dx * math.tan(comp)
    X = [[0.] * nx for _ in range(ny)]
    Y = [[0.] * nx for _ in range(ny)]
    b, continue_b = 3.5, 0.
    for i in range(nx):
        SL = math.sqrt(math.pow(xb[i] - xa[i], 2) + math.pow(yb[i] - ya[i], 2))
        dy = 1. / (ny - 1.)
        delta = q["hy_wall"] / SL
        while True:  # continue_bnew: do { ... } while (|bnew - b| > 1e-6) -- b == bnew here
            fb = (math.exp(b / (ny - 1.)) - 1.) / (math.exp(b) - 1.) - delta
            fbx = (math.exp(b / (ny - 1.)) / (ny - 1.) * (math.exp(b) - 1.) -
                   (math.exp(b / (ny - 1.)) - 1.) * math.exp(b)) / math.pow(math.exp(b) - 1., 2)
            bnew = b - fb / fbx
            b = bnew
            continue_b += 1
            if not continue_b < 10:  # if (continue_b < 10) goto continue_bnew
                break
        a = 1. / (math.exp(b) - 1.)
        for j in range(ny):
            s = j * dy
            sy = a * (math.exp(s * b) - 1)
            X[j][i] = xa[i] + (xb[i] - xa[i]) * sy
            Y[j][i] = ya[i] + (yb[i] - ya[i]) * sy
    bb, Jmax = 3., 20
    for _ in range(10):
        for j in range(1, Jmax):
            ddx, ddy = [0.] * nx, [0.] * nx
            for i in range(1, nx - 1):
                qn = math.sqrt(math.pow(X[j][i + 1] - X[j][i - 1], 2) + math.pow(Y[j][i + 1] - Y[j][i - 1], 2))
                qnx = -(Y[j][i + 1] - Y[j][i - 1]) / qn
                qny = (X[j][i + 1] - X[j][i - 1]) / qn
                s = (X[j][i] - X[j - 1][i]) * qnx + (Y[j][i] - Y[j - 1][i]) * qny
                ddx[i] = s * qnx - (X[j][i] - X[j - 1][i])
                ddy[i] = s * qny - (Y[j][i] - Y[j - 1][i])
            for i in range(1, nx - 1):
                dx1 = (ddx[i - 1] + 2. * ddx[i] + ddx[i + 1]) / 4.
                dy1 = (ddy[i - 1] + 2. * ddy[i] + ddy[i + 1]) / 4.
                X[j][i] = X[j][i] + math.exp(-bb * j / Jmax) / 2. * dx1
                Y[j][i] = Y[j][i] + math.exp(-bb * j / Jmax) / 2. * dy1
    x3 = np.zeros((nz, ny, nx))
    y3, z3 = np.zeros_like(x3), np.zeros_like(x3)
    NPZ = [nz // N + 1 if r < nz % N else nz // N for r in range(N)]
    NP = [0] * N
    for r in range(1, N):
        NP[r] = NP[r - 1] + NPZ[r - 1]
    for r in range(N):
        NZ = NPZ[r]
        for k in range(NZ):
            z = k * Lz * (NPZ[r] - 1) / ((NZ - 1) * (nz - 1)) + NP[r] * Lz / (nz - 1)
            for j in range(ny):
                tmp = X[j][ni - 1]
                for i in range(ni):
                    x3[NP[r] + k, j, i] = (X[j][i] - X[j][0]) * (Li - Lz * math.tan(sw) + Lz / (nz - 1) * (
                        k + NP[r]) * math.tan(sw)) / Li + X[j][0]
                    y3[NP[r] + k, j, i] = Y[j][i]
                    z3[NP[r] + k, j, i] = z
                for i in range(ni, nx):
                    x3[NP[r] + k, j, i] = x3[NP[r] + k, j, ni - 1] + X[j][i] - tmp
                    y3[NP[r] + k, j, i] = Y[j][i]
                    z3[NP[r] + k, j, i] = z
    return x3, y3, z3


@pytest.mark.parametrize("kw", [{}, dict(sw_angle=30.0, nprocs=2), dict(nprocs=3, nz=7, comp_angle=18.0)])
def test_swept_ramp_matches_the_c_program(kw):
    q = dict(SMALL, **kw)
    got = meshgen.swept_ramp_mesh(q)
    ref = _c_program(q)
    for g, r in zip(got, ref):
        assert np.array_equal(g, r)


def test_swept_ramp_geometry(tmp_path):
    q = dict(SMALL)
    x, y, z = meshgen.swept_ramp_mesh(q)
    ni, nc = q["nx_inlet"], q["nx_corner"]
    t = math.tan(math.radians(q["comp_angle"]))
    # the wall: flat before the corner, along the ramp after it
    assert np.all(y[:, 0, :ni] == 0.0)
    xr, yr = x[0, 0, ni + nc // 2 + 1:], y[0, 0, ni + nc // 2 + 1:]
    assert np.allclose(yr, xr * t, rtol=1e-12, atol=1e-12)
    # the first spacing off the wall is hy_wall in the first column (ten Newton steps)
    assert abs(math.hypot(x[0, 1, 0] - x[0, 0, 0], y[0, 1, 0] - y[0, 0, 0]) - q["hy_wall"]) < 1e-9
    # grid lines increase; z spans [0, Lz]
    assert (np.diff(x[0], axis=1) > 0).all() and (np.diff(y[0], axis=0) > 0).all()
    assert z[0].max() == 0.0 and z[-1].min() == pytest.approx(q["lz"], rel=1e-15)
    # the OCFD file round-trips, and the readfort.jl pipeline reads it
    path = str(tmp_path / "OCFD3d-Mesh.dat")
    meshgen.write_ocfd_mesh(path, x, y, z)
    back = read_ocfd_mesh(path, q["nx"], q["ny"], q["nz"])
    assert all(np.array_equal(a, b) for a, b in zip(back, (x, y, z)))
    X, Y, Z = mesh_from_ocfd(path, q["nx"], q["ny"], q["nz"])
    assert X.dtype == np.float32 and np.array_equal(X[NG:-NG, NG:-NG, NG:-NG], (x.astype(np.float32) / np.float32(1000)))
    m, J = meshgen.metrics_f32(X, Y, Z)
    assert np.isfinite(J).all() and (J[NG:-NG, NG:-NG, NG:-NG] > 0).all()
    # the generator's other files: y1d.dat, Tecplot text, the 2-D record file
    x3, y3, z3, x2, y2 = meshgen.swept_ramp_mesh(q, with_2d=True)
    assert np.array_equal(x3, x) and np.array_equal(y2, y[0])
    paths = meshgen.write_swept_outputs(str(tmp_path / "out"), dict(q, tec1=1, mesh2d=1, tec2=1), x3, y3, z3, x2, y2)
    assert [os.path.basename(p) for p in paths] == ["OCFD3d-Mesh.dat", "y1d.dat", "gridxy.dat", "OCFD2d-Mesh.dat",
                                                    "grid.dat"]
    y1d = open(paths[1]).read().splitlines()
    assert len(y1d) == q["ny"] and y1d[1] == "%15.6f" % y2[1, 0]
    txt = open(paths[2]).read().splitlines()
    assert txt[:2] == ["variables=x,y", f"zone i={q['nx']} ,j={q['ny']}"] and len(txt) == 2 + q["nx"] * q["ny"]
    assert txt[2 + q["nx"] + 3] == "%15.6f%15.6f" % (x2[1, 3], y2[1, 3])
    raw = np.fromfile(paths[3], dtype=np.uint8)
    rec = q["nx"] * q["ny"] * 8
    assert raw.size == 2 * (rec + 8) and np.array_equal(raw[4:4 + rec].view("<f8").reshape(x2.shape), x2)
    g = open(paths[4]).read().splitlines()
    assert g[1] == f"zone i={q['nx']} ,j={q['ny']} ,k={q['nz']}" and len(g) == 2 + x3.size
    params = tmp_path / "swept-compression-grid.in"
    params.write_text("nx ny nz Nprocs\n64 24 6 1\nnx_inlet nx_conner nx_buff\n40 20 4\n"
                      "dx_inlet Lx_inlet Lx_conner alfax_buff\n0.9 30. 8. 1.05\nsw_angle comp_angle\n0. 24.\n"
                      "High hy_wall Lz\n6. 0.01 3.\nTecplot2D Mesh2D Tecplot3D\n1 1 0\n")
    r = meshgen.read_swept_params(str(params))
    assert {k: r[k] for k in SMALL} == SMALL
    with pytest.raises(ValueError):
        meshgen.swept_ramp_mesh(q, nx_buff=5)  # parts do not add up to nx
    with pytest.raises(ValueError):
        meshgen.swept_ramp_mesh(q, nprocs=4)  # a process with one plane


def _metric_loops(x, y, z, readfort):
    """readfort.jl:103-181 / parse_mesh.jl:138-248 cell by cell on Julia-ordered [i, j, k]
    arrays, 1-based indices as in the source."""
    f32 = np.float32
    Nxt, Nyt, Nzt = x.shape

    def CD6(f):
        if readfort:
            return f32(1) / f32(60) * (f[6] - f[0]) - f32(3) / f32(20) * (f[5] - f[1]) + f32(3) / f32(4) * (f[4] - f[2])
        return f32(1 / 60 * float(f[6] - f[0]) - 3 / 20 * float(f[5] - f[1]) + 3 / 4 * float(f[4] - f[2]))

    def CD2_L(f):
        if readfort:
            return f32(2) * f[1] - f32(0.5) * f[2] - f32(1.5) * f[0]
        return f32(float(f32(2) * f[1]) - 0.5 * float(f[2]) - 1.5 * float(f[0]))

    def CD2_R(f):
        if readfort:
            return f32(-2) * f[1] + f32(0.5) * f[0] + f32(1.5) * f[2]
        return f32(float(f32(-2) * f[1]) + 0.5 * float(f[0]) + 1.5 * float(f[2]))

    D = {}
    for name, a in (("x", x), ("y", y), ("z", z)):
        for d, n in ((0, Nxt), (1, Nyt), (2, Nzt)):
            out = np.zeros(a.shape, f32)
            for idx in np.ndindex(*a.shape):
                i = idx[d] + 1  # 1-based along d
                line = lambda lo, hi: [a[tuple(idx[:d]) + (t - 1,) + tuple(idx[d + 1:])] for t in range(lo, hi + 1)]
                if 4 <= i <= n - 3:
                    out[idx] = CD6(line(i - 3, i + 3))
                elif i <= 3:
                    out[idx] = CD2_L(line(i, i + 2))
                else:
                    out[idx] = CD2_R(line(i - 2, i))
            D[name + "xez"[d]] = out
    xx, xe, xz = D["xx"], D["xe"], D["xz"]
    yx, ye, yz = D["yx"], D["ye"], D["yz"]
    zx, ze, zz = D["zx"], D["ze"], D["zz"]
    J = f32(1) / (xx * (ye * zz - yz * ze) - xe * (yx * zz - yz * zx) + xz * (yx * ze - ye * zx))
    m = [ye * zz - yz * ze, xz * ze - xe * zz, xe * yz - xz * ye, yz * zx - yx * zz, xx * zz - xz * zx,
         xz * yx - xx * yz, yx * ze - ye * zx, xe * zx - xx * ze, xx * ye - xe * yx]
    return m, J


@pytest.mark.parametrize("coefficients", ["readfort", "parse_mesh"])
def test_metrics_f32_matches_the_julia_loops(coefficients):
    rng = np.random.default_rng(6)
    shape = (9, 10, 11)  # (Nzt, Nyt, Nxt): every cell within three layers of a face somewhere
    k, j, i = np.meshgrid(*[np.arange(s, dtype=np.float64) for s in shape], indexing="ij")
    x = (0.1 * i + 0.01 * np.sin(j + k) + 1e-3 * rng.standard_normal(shape)).astype(np.float32)
    y = (0.2 * j + 0.02 * np.cos(i) + 1e-3 * rng.standard_normal(shape)).astype(np.float32)
    z = (0.3 * k + 0.01 * np.sin(i + j)).astype(np.float32)
    m, J = meshgen.metrics_f32(x, y, z, coefficients)
    mr, Jr = _metric_loops(*[a.transpose(2, 1, 0) for a in (x, y, z)], readfort=coefficients == "readfort")
    assert np.array_equal(J, Jr.transpose(2, 1, 0))
    for a, r in zip(m, mr):
        assert a.dtype == np.float32 and np.array_equal(a, r.transpose(2, 1, 0))


def test_metrics_f32_against_the_oracle_fp64():
    orc = pytest.importorskip("oracle.oracle")
    from flame3d_mhd_gb300.abi import make_params
    from test_gpu_parity import curvilinear_coords
    P = make_params(16, 12, 10)
    x, y, z = curvilinear_coords(P)
    Q0 = np.zeros((6,) + x.shape)
    Q0[0] = 1.0
    Q0[4] = 1.0
    Q0[5] = 1.0 / P.rg
    # the FP64 metrics of the same Float32 coordinates: only the Float32 arithmetic differs.
    # Errors relative to the largest metric (the off-diagonal ones are differences of
    # products as large as the diagonal ones) and to the largest J. readfort.jl sums the
    # CD6 terms in Float32 and loses about 2x to the cancellation between them (measured
    # 2.1e-6 and 2.4e-6, about 17 ulps); parse_mesh.jl sums in FP64 and rounds once
    # (1.9e-7 and 3.3e-7).
    x, y, z = (a.astype(np.float32) for a in (x, y, z))
    m64, J64, _, _ = orc.prepare(P, Q0, *(a.astype(np.float64) for a in (x, y, z)))
    scale = max(np.abs(b).max() for b in m64)
    for coefficients, tol in (("readfort", 5e-6), ("parse_mesh", 1e-6)):
        m, J = meshgen.metrics_f32(x, y, z, coefficients)
        assert max(np.abs(a - b).max() for a, b in zip(m, m64)) <= tol * scale
        assert np.abs(J - J64).max() <= tol * np.abs(J64).max()


def test_flat_plate_and_reference_files(tmp_path):
    X, Y, Z = meshgen.flat_plate_grid(16, 12, 6)
    I = (slice(NG, -NG),) * 3
    assert X.dtype == np.float32 and X.shape == (6 + 2 * NG, 12 + 2 * NG, 16 + 2 * NG)
    assert Y[I].min() == 0.0 and Y[I].max() == np.float32(0.1) and X[I].max() == np.float32(2.0)
    assert (np.diff(Y[I], axis=1) > 0).all() and np.diff(np.diff(Y[NG, NG:-NG, NG])).min() > 0  # finer at the wall
    ref = extend_ghosts(*[np.pad(A[I], NG) for A in (X, Y, Z)], dtype=np.float32, rule="solver")
    assert all(np.array_equal(A, R) for A, R in zip((X, Y, Z), ref))
    pm, pg = meshgen.reference_files(str(tmp_path), X, Y, Z, "parse_mesh")
    with h5.H5File(pm) as f:
        assert f.dataset("J").filters and f.dataset("J").dtype == np.float32
    m, J = files.read_metrics(pm, dtype=np.float32)
    m2, J2 = meshgen.metrics_f32(X, Y, Z, "parse_mesh")
    assert np.array_equal(J, J2) and all(np.array_equal(a, b) for a, b in zip(m, m2))
    Xr, Yr, Zr = files.read_mesh(pg)
    assert np.array_equal(Xr, X) and np.array_equal(Yr, Y) and np.array_equal(Zr, Z)
    # the command line, with parse_mesh.jl's mesh.vts
    assert meshgen.main(["plate", "--nx", "16", "--ny", "12", "--nz", "6", "--out", str(tmp_path / "p"),
                         "--vis"]) == 0
    assert sorted(os.listdir(tmp_path / "p")) == ["mesh.h5", "mesh.vts", "metrics.h5"]
    from flame3d_mhd_gb300 import vtk
    v = vtk.read_vts(str(tmp_path / "p" / "mesh.vts"))
    assert v["extent"] == (16 + 2 * NG, 12 + 2 * NG, 6 + 2 * NG)
    assert np.array_equal(v["J"], J.ravel()) and np.array_equal(v["dedy"], m[4].ravel())
    assert np.array_equal(v["points"][:, 1], Y.ravel())


# ---- pinned on the reference program itself ------------------------------------------------
# tests/golden/swept_ramp_ref.npz holds OCFD3d-Mesh.dat coordinates written by the unmodified
# swept-compression-ramp.c (compiled against the MPI stand-in oracle/ref_ramp/mpi.h; made by
# tests/golden/make_ramp_fixture.py) and digests of its 1000 x 240 x 100 benchmark grid from
# the program built at gcc's default optimisation level and at -O2.
def _ramp_fixture():
    import json
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "swept_ramp_ref.npz"))
    return d, json.loads(str(d["meta"]))


@pytest.mark.parametrize("name", ["one_process", "two_processes_swept", "three_processes"])
def test_swept_ramp_equals_reference_program(name):
    d, meta = _ramp_fixture()
    q = dict(meta["small"], **meta["variants"][name])
    got = meshgen.swept_ramp_mesh(q)
    for a, key in zip(got, "xyz"):
        assert np.array_equal(a, d[f"{name}_{key}"]), key


@pytest.mark.parametrize("square,build", [("libm", "O0"), ("mul", "O2")])
def test_swept_ramp_benchmark_grid_digest(square, build):
    import hashlib
    _, meta = _ramp_fixture()
    h = hashlib.sha256()
    for a in meshgen.swept_ramp_mesh(meta["benchmark"], square=square):
        h.update(np.ascontiguousarray(a, dtype="<f8").tobytes())
    assert h.hexdigest() == meta[f"benchmark_sha256_{build}"]


def test_swept_ramp_live_against_reference_program():
    """Runs the compiled reference program where its source tree is present (oracle/_ref)."""
    from oracle.ref_ramp import run_ref
    if not run_ref.available():
        pytest.skip("the reference program is not built here")
    q = dict(SMALL, nx=48, nx_inlet=30, nx_corner=14, nx_buff=4, ny=22, nz=8, nprocs=2, sw_angle=15.0,
             comp_angle=20.0, hy_wall=0.02)
    for o2, square in ((False, "libm"), (True, "mul")):
        ref = run_ref.run(q, o2=o2)
        got = meshgen.swept_ramp_mesh(q, square=square)
        for a, b in zip(got, ref):
            assert np.array_equal(a, b)
