"""The oracle's finite-volume restatement (FVM.jl) on the CPU: a separate per-face Python
restatement (scalar loops, small grids) against the C++ oracle for both reconstructions and
every branch, free-stream preservation on a Cartesian grid, and conservation on a periodic
curvilinear grid.

Tolerances: 1e-12 relative to the flux scale for the two restatements (same formulas,
different operation order); 1e-13 of the flux scale for free stream and conservation.
Faces whose normal has |ny| = |nz| to rounding are skipped in the cross-check: the tangent
basis of the characteristic fields switches there (FVM.jl:75-79), and which basis a
restatement takes depends on its rounding (the GPU computes normals in the C++ oracle's
operation order, so those two always agree)."""
import math

import numpy as np
import pytest

from flame3d_mhd_gb300.abi import BC_PERIODIC, SCHEME_FVM_CONS, SCHEME_FVM_EIGEN, make_params
from oracle import oracle as orc

NG = 4


def _coords(P, amp, seed=0):
    """Smoothly perturbed periodic-in-index coordinates at every cell (ghosts included)."""
    nzt, nyt, nxt = P.nz + 8, P.ny + 8, P.nx + 8
    k, j, i = np.meshgrid(np.arange(nzt), np.arange(nyt), np.arange(nxt), indexing="ij")
    h = 1.0 / max(P.nx, P.ny, P.nz)
    tp = 2 * np.pi
    X, Y, Z = (i - NG + 0.5) * h, (j - NG + 0.5) * h, (k - NG + 0.5) * h
    x = X + amp * np.sin(tp * Y * 0.7) * np.sin(tp * Z * 0.9)
    y = Y + amp * np.sin(tp * Z * 0.8) * np.sin(tp * X * 1.1)
    z = Z + amp * np.sin(tp * X * 0.6) * np.sin(tp * Y * 1.3)
    return x, y, z


def _state(P, seed, spikes=0, noise=0.3):
    rng = np.random.default_rng(seed)
    shape = (6, P.nz + 8, P.ny + 8, P.nx + 8)
    Q = np.zeros(shape)
    Q[0] = 1.0 + 0.2 * rng.random(shape[1:])
    Q[1:4] = 0.3 * rng.standard_normal((3, *shape[1:]))
    Q[4] = (1.0 / 1.4) * (1.0 + noise * rng.random(shape[1:]))
    if spikes:
        idx = tuple(rng.integers(NG, s - NG, spikes) for s in shape[1:])
        Q[4][idx] *= 3.0
        Q[0][idx] *= 2.0
    Q[5] = Q[4] / (Q[0] * P.rg)
    return Q


# ---- a separate scalar restatement of one face of FVM.jl ---------------------------------
def _minmod(a, b):
    return ((b if abs(a) > abs(b) else a) if a * b > 0 else 0.0)


def _weno7(V, ss):
    V1, V2, V3, V4, V5, V6, V7 = V
    q = [-3 * V1 + 13 * V2 - 23 * V3 + 25 * V4, V2 - 5 * V3 + 13 * V4 + 3 * V5,
         -V3 + 7 * V4 + 7 * V5 - V6, 3 * V4 + 13 * V5 - 5 * V6 + V7]
    IS = [V1 * (547 * V1 - 3882 * V2 + 4642 * V3 - 1854 * V4) + V2 * (7043 * V2 - 17246 * V3 + 7042 * V4)
          + V3 * (11003 * V3 - 9402 * V4) + V4 * (2107 * V4),
          V2 * (267 * V2 - 1642 * V3 + 1602 * V4 - 494 * V5) + V3 * (2843 * V3 - 5966 * V4 + 1922 * V5)
          + V4 * (3443 * V4 - 2522 * V5) + V5 * (547 * V5),
          V3 * (547 * V3 - 2522 * V4 + 1922 * V5 - 494 * V6) + V4 * (3443 * V4 - 5966 * V5 + 1602 * V6)
          + V5 * (2843 * V5 - 1642 * V6) + V6 * (267 * V6),
          V4 * (2107 * V4 - 9402 * V5 + 7042 * V6 - 1854 * V7) + V5 * (11003 * V5 - 17246 * V6 + 4642 * V7)
          + V6 * (7043 * V6 - 3882 * V7) + V7 * (547 * V7)]
    a = [d / (1e-10 + s * ss) ** 2 for d, s in zip((1, 12, 18, 4), IS)]
    return sum(x * y for x, y in zip(a, q)) / sum(a) / 12


def _weno5(V, ss):
    _, a, b, c, d, e, _ = V
    s = [13 * (a - 2 * b + c) ** 2 + 3 * (a - 4 * b + 3 * c) ** 2, 13 * (b - 2 * c + d) ** 2 + 3 * (b - d) ** 2,
         13 * (c - 2 * d + e) ** 2 + 3 * (3 * c - 4 * d + e) ** 2]
    w = [dd / (1e-8 + x * ss) ** 2 for dd, x in zip((1, 6, 3), s)]
    v = [2 * a - 7 * b + 11 * c, -b + 5 * c + 2 * d, 2 * c + 5 * d - e]
    return sum(x * y for x, y in zip(w, v)) / sum(w) / 6


def _side(br, right, V, ss):
    if br == 1:
        return _weno7(V, ss)
    if br == 2:
        return _weno5(V, ss)
    if right:
        return V[3] - 0.5 * _minmod(V[3] - V[2], V[3] - V[4])
    return V[3] + 0.5 * _minmod(V[3] - V[2], V[4] - V[3])


def _hllc(g, UL, UR, n):
    def prim(U):
        r = U[0]
        u = np.array(U[1:4]) / r
        p = (g - 1) * (U[4] - 0.5 * r * u @ u)
        return r, u, U[4], p, math.sqrt(abs(g * p / r)), u @ n

    rL, uL, EL, pL, cL, qL = prim(UL)
    rR, uR, ER, pR, cR, qR = prim(UR)
    sL, sR = math.sqrt(rL), math.sqrt(rR)
    ur = (sL * uL + sR * uR) / (sL + sR)
    Hr = (sL * (EL + pL) / rL + sR * (ER + pR) / rR) / (sL + sR)
    cr = math.sqrt(abs((g - 1) * (Hr - 0.5 * ur @ ur)))
    SL, SR = min(qL - cL, ur @ n - cr), max(qR + cR, ur @ n + cr)
    Ss = (pR - pL + rL * qL * (SL - qL) - rR * qR * (SR - qR)) / (rL * (SL - qL) - rR * (SR - qR) + 1e-12)

    def phys(r, u, E, p, q):
        return np.array([r * q, *(r * u * q + p * n), (E + p) * q])

    def star(U, r, u, E, p, q, S):
        f = r * (S - q) / (S - Ss)
        Us = np.array([f, *(f * (u + (Ss - q) * n)), f * (E / r + (Ss - q) * (Ss + p / (r * (S - q))))])
        return phys(r, u, E, p, q) + S * (Us - np.asarray(U))

    if SL >= 0:
        return phys(rL, uL, EL, pL, qL)
    if SR <= 0:
        return phys(rR, uR, ER, pR, qR)
    if Ss >= 0:
        return star(UL, rL, uL, EL, pL, qL, SL)
    return star(UR, rR, uR, ER, pR, qR, SR)


def _face(P, d, eigen, phi, S, Q, U, x, y, z, i, j, k):
    """Face of direction d between full (0-based) cells (i,j,k) and (i,j,k)+e_d."""
    e = [0, 0, 0]
    e[d] = 1
    a_, b_ = (1, 2) if d == 0 else ((0, 2) if d == 1 else (0, 1))

    def at(A, o, t=(0, 0, 0)):
        c = [i + o * e[0] + t[0], j + o * e[1] + t[1], k + o * e[2] + t[2]]
        return A[..., c[2], c[1], c[0]]

    def tv(sa, sb):
        t = [0, 0, 0]
        t[a_] += sa
        t[b_] += sb
        return tuple(t)

    def corner(A, sa, sb):  # mean of the 8 cells around the corner (+-a/2, +-b/2) of the face
        return sum(at(A, s, tv(pa, pb)) for s in (0, 1) for pa in (0, sa) for pb in (0, sb)) / 8

    d1 = np.array([corner(A, 1, 1) - corner(A, -1, -1) for A in (x, y, z)])
    d2 = np.array([corner(A, -1, 1) - corner(A, 1, -1) for A in (x, y, z)])
    nvec = (-0.5 if d == 1 else 0.5) * np.cross(d1, d2)
    area = math.sqrt(nvec @ nvec + 1e-20)
    n = nvec / area
    phimax = max(at(phi, o) for o in range(-2, 4))
    br = 0 if phimax < P.phi1 else (1 if phimax < P.phi2 else (2 if phimax < P.phi3 else 3))
    lin = np.array([-3, 25, -101, 319, 214, -38, 4]) / 420.0
    VLs = [at(U, o) for o in range(-3, 4)]
    VRs = [at(U, o) for o in range(4, -3, -1)]
    if br == 0:
        UL = sum(c * v for c, v in zip(lin, VLs))
        UR = sum(c * v for c, v in zip(lin, VRs))
    else:
        ss = 2.0 / (at(S, 1) + at(S, 0))
        if not eigen:
            UL = np.array([_side(br, False, [v[m] for v in VLs], ss) for m in range(5)])
            UR = np.array([_side(br, True, [v[m] for v in VRs], ss) for m in range(5)])
        else:
            g = P.gamma
            ql, qr = at(Q, 0), at(Q, 1)
            sl, sr = math.sqrt(ql[0]), math.sqrt(qr[0])
            u = (sl * ql[1:4] + sr * qr[1:4]) / (sl + sr)
            Hs = [g / (g - 1) * q[4] / q[0] + 0.5 * q[1:4] @ q[1:4] for q in (ql, qr)]
            H = (sl * Hs[0] + sr * Hs[1]) / (sl + sr)
            v2 = 0.5 * u @ u
            c = math.sqrt((g - 1) * (H - v2))
            if abs(n[2]) <= abs(n[1]):
                den = math.sqrt(n[0] ** 2 + n[1] ** 2 + 1e-12)
                l = np.array([-n[1] / den, n[0] / den, 0.0])
            else:
                den = math.sqrt(n[0] ** 2 + n[2] ** 2 + 1e-12)
                l = np.array([-n[2] / den, 0.0, n[0] / den])
            mm = np.cross(n, l)
            K = g - 1
            un, ul, um = u @ n, u @ l, u @ mm
            Lm = np.array([[0.5 * (K * v2 / c ** 2 + un / c), *(-0.5 * (K * u / c ** 2 + n / c)), 0.5 * K / c ** 2],
                           [1 - K * v2 / c ** 2, *(K * u / c ** 2), -K / c ** 2],
                           [0.5 * (K * v2 / c ** 2 - un / c), *(-0.5 * (K * u / c ** 2 - n / c)), 0.5 * K / c ** 2],
                           [-ul, *l, 0.0], [-um, *mm, 0.0]])
            Rm = np.array([[1, *(u - n * c), H - un * c], [1, *u, v2], [1, *(u + n * c), H + un * c],
                           [0, *l, ul], [0, *mm, um]])
            UL, UR = np.zeros(5), np.zeros(5)
            for fld in range(5):
                vl = _side(br, False, [Lm[fld] @ v for v in VLs], ss)
                vr = _side(br, True, [Lm[fld] @ v for v in VRs], ss)
                UL += Rm[fld] * vl
                UR += Rm[fld] * vr
    return _hllc(P.gamma, UL, UR, n) * area, br, abs(abs(n[1]) - abs(n[2]))


@pytest.mark.parametrize("eigen", [True, False])
def test_fvm_oracle_matches_scalar_restatement(eigen):
    per = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(7, 6, 5, bc=per, viscous=0, phi1=0.02, phi2=0.1, phi3=0.4,
                    scheme=SCHEME_FVM_EIGEN if eigen else SCHEME_FVM_CONS)
    x, y, z = _coords(P, 0.03)
    Q = _state(P, 11, spikes=12, noise=0.03)
    m, J, Q, U = orc.prepare(P, Q, x, y, z)
    phi = orc.sensor(P, Q)
    seen = set()
    for d in range(3):
        S = orc.metric_norm(P, m[3 * d], m[3 * d + 1], m[3 * d + 2])
        F, br = orc.fvm_face_flux(P, d, eigen, phi, S, Q, U, x, y, z, with_branch=True)
        scale = np.abs(F).max(axis=(1, 2, 3))
        fz, fy, fx = F.shape[1:]
        for kf in range(fz):
            for jf in range(fy):
                for ifc in range(fx):
                    i, j, k = ifc + NG, jf + NG, kf + NG
                    if d == 0: i -= 1
                    if d == 1: j -= 1
                    if d == 2: k -= 1
                    ref, b, tie = _face(P, d, eigen, phi, S, Q, U, x, y, z, i, j, k)
                    assert b == br[kf, jf, ifc]
                    seen.add(b)
                    if eigen and b != 0 and tie < 1e-13:
                        continue
                    assert np.all(np.abs(F[:, kf, jf, ifc] - ref) <= 1e-12 * scale), (d, i, j, k, b)
    assert seen == {0, 1, 2, 3}


@pytest.mark.parametrize("scheme", [SCHEME_FVM_EIGEN, SCHEME_FVM_CONS])
def test_fvm_free_stream_on_cartesian_grid(scheme):
    per = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(8, 7, 6, bc=per, viscous=1, scheme=scheme, phi1=0.0, phi2=1.0, phi3=10.0)
    x, y, z = _coords(P, 0.0)
    Q = np.zeros((6, P.nz + 8, P.ny + 8, P.nx + 8))
    Q[0], Q[1], Q[2], Q[3], Q[4] = 1.2, 0.3, -0.2, 0.1, 0.9
    Q[5] = Q[4] / (Q[0] * P.rg)
    m, J, Q, U = orc.prepare(P, Q, x, y, z)
    orc.set_coordinates(x, y, z)
    try:
        r = orc.rhs(P, Q, m, J)
    finally:
        orc.set_coordinates(None)
    I = (slice(None), slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    flux = 1.2 * 0.3 ** 2 + 0.9  # largest flux component, per unit area
    assert np.abs(r[I]).max() <= 1e-13 * flux * J.max()


@pytest.mark.parametrize("scheme", [SCHEME_FVM_EIGEN, SCHEME_FVM_CONS])
def test_fvm_periodic_conservation(scheme):
    per = [dict(kind=BC_PERIODIC)] * 6
    P = make_params(8, 6, 6, bc=per, viscous=0, scheme=scheme, phi1=0.02, phi2=0.1, phi3=0.4)
    x, y, z = _coords(P, 0.0)
    Q = _state(P, 5, spikes=6)
    m, J, Q, U = orc.prepare(P, Q, x, y, z)
    orc.set_coordinates(x, y, z)
    try:
        r = orc.rhs(P, Q, m, J)
    finally:
        orc.set_coordinates(None)
    I = (slice(NG, -NG), slice(NG, -NG), slice(NG, -NG))
    for n in range(5):
        tot = float((r[n][I] / J[I]).sum())
        assert abs(tot) <= 1e-13 * float(np.abs(r[n][I] / J[I]).sum()), (n, tot)
