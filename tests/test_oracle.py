"""CPU tests of the oracle: known-answer properties of the reference's scheme, a second
independent NumPy restatement, the reference's own Float32 precision, and the committed
golden fixtures. No GPU needed."""
import numpy as np
import pytest

from conftest import rel_linf
from flame3d_mhd_gb300 import cases
from flame3d_mhd_gb300.abi import (BC_PERIODIC, BC_ZERO_GRADIENT, make_params)
from oracle import np_oracle as npo
from oracle import oracle as orc

NG = 4
PER = [dict(kind=BC_PERIODIC)] * 6


def curvi(P, amp=0.03):
    s = (P.nz + 8, P.ny + 8, P.nx + 8)
    ax = [(np.arange(n) - NG + 0.5) / (n - 8) for n in s]
    Z, E, X = np.meshgrid(*ax, indexing="ij")
    tp = 2 * np.pi
    return (X + amp * np.sin(tp * E) * np.sin(tp * Z), E + amp * np.sin(tp * Z) * np.sin(tp * X),
            Z + amp * np.sin(tp * X) * np.sin(tp * E))


def state(P, seed, spikes=0):
    rng = np.random.default_rng(seed)
    s = (P.nz + 8, P.ny + 8, P.nx + 8)
    Q = np.zeros((6, *s))
    k, j, i = np.meshgrid(*[np.arange(n) for n in s], indexing="ij")
    Q[0] = 1.0 + 0.2 * np.sin(0.3 * i + 0.2 * j) * np.cos(0.25 * k) + 0.02 * rng.uniform(-1, 1, s)
    Q[1] = 0.3 * np.sin(0.2 * j + 0.1 * k) + 0.05 * rng.uniform(-1, 1, s)
    Q[2] = 0.2 * np.cos(0.3 * i) + 0.05 * rng.uniform(-1, 1, s)
    Q[3] = -0.1 * np.sin(0.15 * i + 0.3 * k) + 0.05 * rng.uniform(-1, 1, s)
    Q[4] = (1.0 + 0.2 * np.cos(0.2 * i - 0.3 * j + 0.1 * k)) / 1.4 + 0.01 * rng.uniform(-1, 1, s)
    for _ in range(spikes):
        a, b, c = [int(rng.integers(NG, n - NG)) for n in s]
        Q[4, a, b, c] *= float(rng.uniform(5, 200))
    Q[5] = Q[4] / (Q[0] * P.rg)
    return Q


def prepared(P, seed=1, spikes=0, amp=0.03):
    x, y, z = curvi(P, amp)
    return orc.prepare(P, state(P, seed, spikes), x, y, z)


# ------------------------------------------------------------------------- known answers
@pytest.mark.parametrize("split", ["SW", "LF", "VL", "AUSM"])
def test_split_sums_to_physical_flux(split):
    """Fp + Fm = F(Q) . A for every splitter (an identity of split.jl)."""
    P = make_params(8, 6, 5, split=split, bc=PER)
    m, J, Q, U = prepared(P, seed=2)
    for d in range(3):
        A = m[3 * d:3 * d + 3]
        S = orc.metric_norm(P, *A)
        Fp, Fm = orc.split(P, Q, *A, S)
        rho, u, v, w, p, T = Q
        un = A[0] * u + A[1] * v + A[2] * w
        E = p / (P.gamma - 1) + 0.5 * rho * (u * u + v * v + w * w)
        F = np.stack([rho * un, rho * u * un + A[0] * p, rho * v * un + A[1] * p, rho * w * un + A[2] * p,
                      (E + p) * un])
        assert rel_linf(Fp + Fm, F) <= 1e-13


@pytest.mark.parametrize("character", [0, 1])
@pytest.mark.parametrize("split", ["SW", "LF", "VL", "AUSM"])
def test_free_stream_preserved_on_cartesian_grid(character, split):
    c = cases.tgv(12, character=character, split=split)
    P = c["params"]
    P.phi1, P.phi2, P.phi3 = 0.02, 0.1, 0.4  # hybrid switch active
    Q0 = c["Q"].copy()
    I = (slice(NG, -NG),) * 3
    for n, val in enumerate([1.2, 0.3, -0.2, 0.1, 0.9, 0.9 / (1.2 * P.rg)]):
        Q0[n][I] = val
    m, J, Q, U = orc.prepare(P, Q0, c["x"], c["y"], c["z"])
    r = orc.rhs(P, Q, m, J)
    assert np.abs(r).max() <= 1e-13


def periodic_images(a):
    """Overwrite the ghost layers of a (Nz+8, Ny+8, Nx+8) array with periodic images."""
    out = a.copy()
    for ax in range(3):
        n = a.shape[ax] - 2 * NG
        idx = (np.arange(a.shape[ax]) - NG) % n + NG
        out = np.take(out, idx, axis=ax)
    return np.ascontiguousarray(out)


@pytest.mark.parametrize("character", [0, 1])
def test_periodic_conservation(character):
    """Sum over cells of RHS/J telescopes to zero on an all-periodic curvilinear grid whose
    ghost metrics are periodic images (div.jl). The reference's own metric recipe uses
    one-sided CD2 in the outer ghost layers (parse_mesh.jl:200-235), which is not periodic;
    the property tested here is the scheme's telescoping, so the metrics are made periodic."""
    P = make_params(12, 10, 8, character=character, phi1=0.02, phi2=0.1, phi3=0.4, viscous=1, rg=1.0,
                    c_s=1e-2, t_s=1.0, bc=PER)
    m, J, Q, U = prepared(P, seed=3, spikes=10)
    m = [periodic_images(a) for a in m]
    J = periodic_images(J)
    r = orc.rhs(P, Q, m, J)
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    tot = (r[I] / J[I[1:]]).sum(axis=(1, 2, 3))
    scale = np.abs(r[I] / J[I[1:]]).sum(axis=(1, 2, 3))
    assert (np.abs(tot) <= 1e-12 * scale).all()


def test_axis_permutation_symmetry_componentwise():
    """Swapping x and y of a component-wise problem swaps the RHS (up to summation order)."""
    P = make_params(10, 10, 8, character=0, phi1=0.02, phi2=0.1, phi3=0.4, bc=PER)
    s = (P.nz + 8, P.ny + 8, P.nx + 8)
    ax = (np.arange(10 + 8) - NG + 0.5) / 10
    az = (np.arange(8 + 8) - NG + 0.5) / 8
    Z, Y, X = np.meshgrid(az, ax, ax, indexing="ij")
    Q0 = state(P, 5, spikes=5)
    m, J, Q, U = orc.prepare(P, Q0, X, Y, Z)
    r = orc.rhs(P, Q, m, J)
    # swap x <-> y: transpose the two last axes, swap u and v, swap the metric roles
    Qs = Q0.transpose(0, 1, 3, 2).copy()
    Qs[[1, 2]] = Qs[[2, 1]]
    ms, Js, Qp, Up = orc.prepare(P, np.ascontiguousarray(Qs), X, Y, Z)
    rs = orc.rhs(P, Qp, ms, Js)
    back = rs.transpose(0, 1, 3, 2).copy()
    back[[1, 2]] = back[[2, 1]]
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    assert rel_linf(back[I], r[I]) <= 1e-13


@pytest.mark.parametrize("scheme,order", [("up7", 7), ("weno5", 5)])
def test_order_of_accuracy(scheme, order):
    """Density wave advected at constant velocity and pressure: d(rho)/dt = -u d(rho)/dx."""
    errs = []
    for n in (16, 32):
        P = make_params(n, 4, 4, viscous=0, character=0, bc=PER)
        P.phi1, P.phi2, P.phi3 = (np.inf, np.inf, np.inf) if scheme == "up7" else (0.0, 0.0, np.inf)
        h = 1.0 / n
        xa = (np.arange(n + 8) - NG + 0.5) * h
        ya = (np.arange(4 + 8) - NG + 0.5) * 0.25
        Z, Y, X = np.meshgrid(ya, ya, xa, indexing="ij")
        Q0 = np.zeros((6, *X.shape))
        Q0[0] = 1.0 + 0.1 * np.sin(2 * np.pi * X)
        Q0[1] = 0.5
        Q0[4] = 1.0
        Q0[5] = Q0[4] / (Q0[0] * P.rg)
        m, J, Q, U = orc.prepare(P, Q0, X, Y, Z)
        r = orc.rhs(P, Q, m, J)
        exact = -0.5 * 0.1 * 2 * np.pi * np.cos(2 * np.pi * X)
        I = (slice(NG, -NG),) * 3
        errs.append(np.abs(r[0][I] - exact[I]).max())
    rate = np.log2(errs[0] / errs[1])
    assert rate >= order - 0.7, (errs, rate)


def exact_sod(x, t, g=1.4, rl=1.0, pl=1.0, rr=0.125, pr=0.1, x0=0.5):
    """Exact Riemann solution of the Sod problem (density) at time t."""
    cl, cr = np.sqrt(g * pl / rl), np.sqrt(g * pr / rr)
    def f(p, rk, pk, ck):
        if p > pk:
            A, B = 2 / ((g + 1) * rk), (g - 1) / (g + 1) * pk
            return (p - pk) * np.sqrt(A / (p + B))
        return 2 * ck / (g - 1) * ((p / pk) ** ((g - 1) / (2 * g)) - 1)
    lo, hi = 1e-6, 5.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if f(mid, rl, pl, cl) + f(mid, rr, pr, cr) > 0:
            hi = mid
        else:
            lo = mid
    ps = 0.5 * (lo + hi)
    us = 0.5 * (f(ps, rr, pr, cr) - f(ps, rl, pl, cl))
    rsl = rl * (ps / pl) ** (1 / g)
    rsr = rr * ((ps / pr + (g - 1) / (g + 1)) / ((g - 1) / (g + 1) * ps / pr + 1))
    S = np.sqrt(g * pr / rr * ((g + 1) / (2 * g) * ps / pr + (g - 1) / (2 * g)))
    xs = (x - x0) / t
    csl = cl * (ps / pl) ** ((g - 1) / (2 * g))
    rho = np.where(xs < -cl, rl, 0.0)
    fan = (xs >= -cl) & (xs < us - csl)
    rho = np.where(fan, rl * (2 / (g + 1) + (g - 1) / ((g + 1) * cl) * (0 - xs)) ** (2 / (g - 1)), rho)
    rho = np.where((xs >= us - csl) & (xs < us), rsl, rho)
    rho = np.where((xs >= us) & (xs < S), rsr, rho)
    rho = np.where(xs >= S, rr, rho)
    return rho


def test_sod_against_exact_riemann_solution():
    n = 200
    P = make_params(n, 4, 4, viscous=0, bc=[dict(kind=BC_ZERO_GRADIENT)] * 2 + PER[:4])
    h = 1.0 / n
    xa = (np.arange(n + 8) - NG + 0.5) * h
    ya = (np.arange(12) - NG + 0.5) * 0.25
    Z, Y, X = np.meshgrid(ya, ya, xa, indexing="ij")
    Q0 = np.zeros((6, *X.shape))
    left = X < 0.5
    Q0[0] = np.where(left, 1.0, 0.125)
    Q0[4] = np.where(left, 1.0, 0.1)
    Q0[5] = Q0[4] / (Q0[0] * P.rg)
    m, J, Q, U = orc.prepare(P, Q0, X, Y, Z)
    dt, t_end = 0.4 * h / 1.2, 0.2
    steps = int(round(t_end / dt))
    Un = np.zeros_like(U)
    orc.rk3(P, steps, dt, U, Un, Q, m, J)
    rho = Q[0, NG + 1, NG + 1, NG:-NG]
    ex = exact_sod(xa[NG:-NG], steps * dt)
    l1 = np.abs(rho - ex).mean()
    assert l1 < 6e-3, l1
    assert np.isfinite(Q).all()


def test_branch_map_covers_every_scheme():
    P = make_params(16, 12, 10, phi1=0.02, phi2=0.1, phi3=0.4, bc=PER)
    m, J, Q, U = prepared(P, seed=8, spikes=30)
    _, br = orc.rhs(P, Q, m, J, with_branches=True)
    for b in br:
        assert (np.bincount(b.ravel(), minlength=4) > 0).all()


def test_reference_float32_precision_is_far_from_fp64():
    """The reference's own arithmetic (Float32, FP64 WENO7 alphas) differs from FP64 at the
    1e-7..1e-4 level: the reason an FP64 drop-in cannot be bit-faithful to Float32 results."""
    P = make_params(12, 10, 8, phi1=0.02, phi2=0.1, phi3=0.4, bc=PER)
    m, J, Q, U = prepared(P, seed=9, spikes=5)
    r = orc.rhs(P, Q, m, J)
    r32 = orc.rhs32(P, Q.astype(np.float32), [a.astype(np.float32) for a in m], J.astype(np.float32))
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    err = rel_linf(r32[I].astype(np.float64), r[I])
    assert 1e-8 < err < 1e-2


# ------------------------------------------------------------------------- NumPy restatement
@pytest.mark.parametrize("split", ["SW", "LF", "VL", "AUSM"])
def test_numpy_split_matches(split):
    P = make_params(8, 6, 5, split=split, bc=PER)
    m, J, Q, U = prepared(P, seed=10)
    for d in range(3):
        A = m[3 * d:3 * d + 3]
        S = orc.metric_norm(P, *A)
        Fp, Fm = orc.split(P, Q, *A, S)
        Fp2, Fm2 = npo.split(P, Q, *A, S)
        assert rel_linf(Fp2, Fp) <= 1e-14
        assert rel_linf(Fm2, Fm) <= 1e-14


def test_numpy_sensor_matches():
    P = make_params(8, 6, 5, bc=PER)
    m, J, Q, U = prepared(P, seed=11, spikes=5)
    assert rel_linf(npo.sensor(Q)[None], orc.sensor(P, Q)[None]) <= 1e-15


@pytest.mark.parametrize("character", [0, 1])
@pytest.mark.parametrize("split", ["SW", "AUSM"])
def test_numpy_face_flux_and_divergence_match(character, split):
    P = make_params(12, 10, 8, split=split, character=character, phi1=0.02, phi2=0.1, phi3=0.4, viscous=1,
                    rg=1.0, c_s=1e-2, t_s=1.0, bc=PER)
    m, J, Q, U = prepared(P, seed=12, spikes=20)
    phi = orc.sensor(P, Q)
    F = []
    for d in range(3):
        A = m[3 * d:3 * d + 3]
        S = orc.metric_norm(P, *A)
        Fp, Fm = orc.split(P, Q, *A, S)
        Fo = orc.face_flux(P, d, phi, S, Fp, Fm, Q, *A)
        Fn = npo.face_flux(P, d, phi, S, Fp, Fm, Q, *A)
        assert rel_linf(Fn, Fo) <= 1e-13, d
        F.append(Fo)
    Fv = orc.viscous(P, Q, m, J)
    ro = orc.divergence(P, F[0], F[1], F[2], Fv, J)
    rn = npo.divergence(P, F, J, Fv)
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    assert rel_linf(rn[I], ro[I]) <= 1e-13


# ------------------------------------------------------------------------- golden fixtures
def test_golden_fixtures():
    """Fixtures written by tests/golden/make_golden.py with the NumPy restatement."""
    import json
    from pathlib import Path
    gdir = Path(__file__).resolve().parent / "golden"
    files = [f for f in sorted(gdir.glob("*.npz")) if "rhs" in np.load(f).files]  # RHS fixtures only
    assert files, "no golden fixtures"
    for f in files:
        g = np.load(f)
        meta = json.loads(str(g["meta"]))
        P = make_params(*meta["n"], **meta["params"])
        m = [np.ascontiguousarray(g["metrics"][k]) for k in range(9)]
        r = orc.rhs(P, np.ascontiguousarray(g["Q"]), m, np.ascontiguousarray(g["J"]))
        I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
        assert rel_linf(r[I], g["rhs"][I]) <= meta["tol"], f.name


def test_linear_scheme_coefficients_from_the_reference_script():
    """UP7 and CD6 (run.jl:75-77) in the NumPy oracle, the C++ oracle and the CUDA library
    equal the face coefficients the reference's Utils/FDMcoeffs.py derives (fixture made by
    tests/golden/make_fdm_coeffs.py; the script's linear solve rounds at 1e-15)."""
    import json
    import re
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    g = json.loads((root / "tests" / "golden" / "fdm_coeffs.json").read_text())
    up7, cd6 = np.array(g["up7"]), np.array(g["cd6"])
    assert np.abs(npo.UP7 - up7).max() < 2e-15 and np.abs(npo.CD6 - cd6).max() < 2e-15
    P = make_params(8, 8, 8, linear_phi=0.5)
    assert np.abs(npo.consts(P)[2] - np.array(g["blend_half"])).max() < 2e-15
    for src in ("flame3d_mhd_gb300/csrc/api.cu", "oracle/f3d_oracle.hpp"):
        text = (root / src).read_text()
        for name, want in (("up7", up7), ("cd6", cd6)):
            body = re.search(r"const double %s\[7\] = \{([^}]*)\}" % name, text).group(1)
            vals = []
            for t in body.split(","):
                m = re.fullmatch(r"\s*([-+]?[\d.]+)\s*/\s*([\d.]+)\s*", t)
                vals.append(float(m.group(1)) / float(m.group(2)) if m else float(t))
            assert np.abs(np.array(vals) - want).max() < 2e-15, (src, name)
