"""Second, independent restatement of the splitting, reconstruction and divergence in NumPy.

TEST INFRASTRUCTURE ONLY. Vectorised over whole arrays (a different operation order from
the C++ oracle), for grids of at most ~16^3: it cross-checks the C++ oracle and produces
the golden fixtures in tests/golden/. Arrays are (nvar, Nz+8, Ny+8, Nx+8) float64.

  split(method, ...)          split.jl:2-255
  sensor(Q)                   schemes.jl:1-24
  face_flux(...)              schemes.jl:86-288 (component-wise), 700-1012 (characteristic)
  divergence(...)             div.jl:1-50
  metrics(x, y, z)            parse_mesh.jl:139-248
  rhs(P, Q, x, y, z)          the composition, inviscid
"""
from __future__ import annotations

import numpy as np

NG = 4
UP7 = np.array([-3, 25, -101, 319, 214, -38, 4]) / 420.0
CD6 = np.array([0.0, 1 / 60, -2 / 15, 37 / 60, 37 / 60, -2 / 15, 1 / 60])


def consts(P):
    g, rg = P.gamma, P.rg
    lin = UP7 * P.linear_phi + CD6 * (1.0 - P.linear_phi)
    return g, rg, lin


def split(P, Q, A1, A2, A3, S):
    """Fp, Fm at every cell for one metric row (split.jl)."""
    g, rg, _ = consts(P)
    rho, u, v, w, p, T = Q
    m = P.split_method
    if m == 0:  # Steger-Warming, split.jl:2-68
        c = np.sqrt(g * rg * T)
        E1 = A1 * u + A2 * v + A3 * w
        E = [E1, E1 - c * S, E1 + c * S]
        a1, a2, a3 = A1 / S, A2 / S, A3 / S
        Ep = [np.maximum(e, 0.0) for e in E]
        Em = [np.minimum(e, 0.0) for e in E]
        uc = [(u - c * a1, v - c * a2, w - c * a3), (u + c * a1, v + c * a2, w + c * a3)]
        vv = (g - 1) * (u * u + v * v + w * w)
        vvc = [0.5 * (x * x + y * y + z * z) for x, y, z in uc]
        W2 = (3 - g) / (2 * (g - 1)) * c * c
        t1 = rho / (2 * g)
        out = []
        for e in (Ep, Em):
            out.append(np.stack([
                t1 * (2 * (g - 1) * e[0] + e[1] + e[2]),
                t1 * (2 * (g - 1) * e[0] * u + e[1] * uc[0][0] + e[2] * uc[1][0]),
                t1 * (2 * (g - 1) * e[0] * v + e[1] * uc[0][1] + e[2] * uc[1][1]),
                t1 * (2 * (g - 1) * e[0] * w + e[1] * uc[0][2] + e[2] * uc[1][2]),
                t1 * (e[0] * vv + e[1] * vvc[0] + e[2] * vvc[1] + W2 * (e[1] + e[2]))]))
        return out[0], out[1]
    c = np.sqrt(g * p / rho)
    un = A1 * u + A2 * v + A3 * w
    kin = u * u + v * v + w * w
    if m == 1:  # local Lax-Friedrichs, split.jl:70-108
        l0 = np.abs(un) + c * S
        E0 = p / (g - 1) + 0.5 * rho * kin
        F = np.stack([rho * un, rho * u * un + A1 * p, rho * v * un + A2 * p, rho * w * un + A3 * p, (E0 + p) * un])
        Uc = np.stack([rho, rho * u, rho * v, rho * w, E0])
        return 0.5 * (F + l0 * Uc), 0.5 * (F - l0 * Uc)
    M = un / (c * S)
    if m == 2:  # van Leer, split.jl:110-183
        E0 = p / (g - 1) + 0.5 * rho * kin
        F = np.stack([rho * un, rho * u * un + A1 * p, rho * v * un + A2 * p, rho * w * un + A3 * p, (E0 + p) * un])
        unn = un / S
        f1p = rho * c * 0.25 * (M + 1) ** 2 * S
        f1m = -rho * c * 0.25 * (M - 1) ** 2 * S
        t1 = (-unn + 2 * c) / (g * S)
        t2 = (-unn - 2 * c) / (g * S)
        t3 = 1 / (2 * (g * g - 1))
        t4 = 0.5 * (kin - unn * unn)
        sp = np.stack([f1p, f1p * (A1 * t1 + u), f1p * (A2 * t1 + v), f1p * (A3 * t1 + w),
                       f1p * (((g - 1) * unn + 2 * c) ** 2 * t3 + t4)])
        sm = np.stack([f1m, f1m * (A1 * t2 + u), f1m * (A2 * t2 + v), f1m * (A3 * t2 + w),
                       f1m * (((g - 1) * unn - 2 * c) ** 2 * t3 + t4)])
    else:  # AUSM, split.jl:185-255
        h = g * p / (rho * (g - 1)) + 0.5 * kin
        F = np.stack([rho * un, rho * u * un + A1 * p, rho * v * un + A2 * p, rho * w * un + A3 * p, rho * h * un])
        fp = 0.25 * (M + 1) ** 2 * rho * c * S
        fm = -0.25 * (M - 1) ** 2 * rho * c * S
        Pp = p * (0.25 * (M + 1) ** 2 * (2 - M))
        Pm = p * (0.25 * (M - 1) ** 2 * (2 + M))
        sp = np.stack([fp, fp * u + A1 * Pp, fp * v + A2 * Pp, fp * w + A3 * Pp, fp * h])
        sm = np.stack([fm, fm * u + A1 * Pm, fm * v + A2 * Pm, fm * w + A3 * Pm, fm * h])
    Fp = np.where(M <= -1, 0.0, np.where(M >= 1, F, sp))
    Fm = np.where(M <= -1, F, np.where(M >= 1, 0.0, sm))
    return Fp, Fm


def sensor(Q):
    """phi at cells 2..Nt-1 (1-based), zero elsewhere (schemes.jl:1-24)."""
    p = Q[4]
    phi = np.zeros_like(p)
    c = (slice(1, -1),) * 3
    tot = 0.0
    for ax in range(3):  # x, y, z = array axes 2, 1, 0
        a = 2 - ax
        lo = [slice(1, -1)] * 3
        hi = [slice(1, -1)] * 3
        lo[a] = slice(0, -2)
        hi[a] = slice(2, None)
        p1, p2, p3 = p[tuple(lo)], p[c], p[tuple(hi)]
        tot = tot + np.abs(-p1 + 2 * p2 - p3) / (p1 + 2 * p2 + p3)
    phi[c] = tot
    return phi


def _weno7(V, s0):
    V1, V2, V3, V4, V5, V6, V7 = V
    q = [-3 * V1 + 13 * V2 - 23 * V3 + 25 * V4, V2 - 5 * V3 + 13 * V4 + 3 * V5, -V3 + 7 * V4 + 7 * V5 - V6,
         3 * V4 + 13 * V5 - 5 * V6 + V7]
    IS = [V1 * (547 * V1 - 3882 * V2 + 4642 * V3 - 1854 * V4) + V2 * (7043 * V2 - 17246 * V3 + 7042 * V4)
          + V3 * (11003 * V3 - 9402 * V4) + V4 * (2107 * V4),
          V2 * (267 * V2 - 1642 * V3 + 1602 * V4 - 494 * V5) + V3 * (2843 * V3 - 5966 * V4 + 1922 * V5)
          + V4 * (3443 * V4 - 2522 * V5) + V5 * (547 * V5),
          V3 * (547 * V3 - 2522 * V4 + 1922 * V5 - 494 * V6) + V4 * (3443 * V4 - 5966 * V5 + 1602 * V6)
          + V5 * (2843 * V5 - 1642 * V6) + V6 * (267 * V6),
          V4 * (2107 * V4 - 9402 * V5 + 7042 * V6 - 1854 * V7) + V5 * (11003 * V5 - 17246 * V6 + 4642 * V7)
          + V6 * (7043 * V6 - 3882 * V7) + V7 * (547 * V7)]
    d = [1.0, 12.0, 18.0, 4.0]
    a = [dk / (1e-20 + ISk * s0) ** 2 for dk, ISk in zip(d, IS)]
    return sum(ak * qk for ak, qk in zip(a, q)) / sum(a)


def _weno5(V, s0):
    V1, V2, V3, V4, V5 = V
    s = [13 * (V1 - 2 * V2 + V3) ** 2 + 3 * (V1 - 4 * V2 + 3 * V3) ** 2,
         13 * (V2 - 2 * V3 + V4) ** 2 + 3 * (V2 - V4) ** 2,
         13 * (V3 - 2 * V4 + V5) ** 2 + 3 * (3 * V3 - 4 * V4 + V5) ** 2]
    a = [dk / (1e-16 + sk * s0) ** 2 for dk, sk in zip((1.0, 6.0, 3.0), s)]
    v = [2 * V1 - 7 * V2 + 11 * V3, -V2 + 5 * V3 + 2 * V4, 2 * V3 + 5 * V4 - V5]
    return sum(ak * vk for ak, vk in zip(a, v)) / sum(a)


def _minmod(a, b):
    return np.where(a * b > 0, np.where(np.abs(a) > np.abs(b), b, a), 0.0)


def _along(a, d):
    """View with the sweep direction first: (..., N_d-axis, t1, t2) -> axis order (d, other, other)."""
    ax = 2 - d + (a.ndim - 3)
    return np.moveaxis(a, ax, a.ndim - 3)


def face_flux(P, d, phi, S, Fp, Fm, Q, A1, A2, A3):
    """Face flux of direction d in the shape of Fx/Fy/Fz, (5, faces...)."""
    g, rg, lin = consts(P)
    N = [P.nx, P.ny, P.nz][d]
    # interior transverse cells, all cells along d; move d to the leading spatial axis
    sl = [slice(NG, -NG)] * 3
    sl[2 - d] = slice(None)
    sl = tuple(sl)
    fp, fm, q = _along(Fp[(slice(None),) + sl], d), _along(Fm[(slice(None),) + sl], d), _along(Q[(slice(None),) + sl], d)
    ph, s = _along(phi[sl], d), _along(S[sl], d)
    a1, a2, a3 = (_along(x[sl], d) for x in (A1, A2, A3))
    out = []
    for f in range(N + 1):
        r = f + NG  # 0-based full index of the cell right of face f
        pm = ph[r - 3:r + 3].max(axis=0)
        s0 = 2.0 / (s[r - 1] + s[r])
        br = np.where(pm < P.phi1, 0, np.where(pm < P.phi2, 1, np.where(pm < P.phi3, 2, 3)))
        P7 = [fp[:, r - 4 + k] for k in range(7)]
        M7 = [fm[:, r + 3 - k] for k in range(7)]
        up7 = sum(lin[k] * P7[k] for k in range(7)) + sum(lin[k] * M7[k] for k in range(7))
        nnd = (fp[:, r - 1] + 0.5 * _minmod(fp[:, r] - fp[:, r - 1], fp[:, r - 1] - fp[:, r - 2])
               + fm[:, r] - 0.5 * _minmod(fm[:, r + 1] - fm[:, r], fm[:, r] - fm[:, r - 1]))
        if not P.character:
            w7 = (_weno7(P7, s0) + _weno7(M7, s0)) / 12.0
            w5 = (_weno5(P7[1:6], s0) + _weno5(M7[1:6], s0)) / 6.0
        else:
            u, v, w, T = (0.5 * (q[k, r] + q[k, r - 1]) for k in (1, 2, 3, 5))
            nx, ny, nz = (0.5 * (x[r] + x[r - 1]) * s0 for x in (a1, a2, a3))
            first = np.abs(nz) <= np.abs(ny)
            with np.errstate(divide="ignore"):  # np.where evaluates both branches
                ss = np.where(first, 1 / np.sqrt(nx * nx + ny * ny), 1 / np.sqrt(nx * nx + nz * nz))
            lx = np.where(first, -ny * ss, -nz * ss)
            ly = np.where(first, nx * ss, 0.0)
            lz = np.where(first, 0.0, nx * ss)
            mx, my, mz = ny * lz - nz * ly, nz * lx - nx * lz, nx * ly - ny * lx
            qn, ql, qm = u * nx + v * ny + w * nz, u * lx + v * ly + w * lz, u * mx + v * my + w * mz
            q2 = 0.5 * (u * u + v * v + w * w)
            c = np.sqrt(g * rg * T)
            c2, K = 1 / (2 * c), (g - 1) / c ** 2
            K2, H = 0.5 * K, c ** 2 / (g - 1) + q2
            L = [[K2 * q2 + qn * c2, -(K2 * u + nx * c2), -(K2 * v + ny * c2), -(K2 * w + nz * c2), K2],
                 [1 - K * q2, K * u, K * v, K * w, -K],
                 [K2 * q2 - qn * c2, -(K2 * u - nx * c2), -(K2 * v - ny * c2), -(K2 * w - nz * c2), K2],
                 [-ql, lx, ly, lz, 0.0], [-qm, mx, my, mz, 0.0]]
            R = [[1.0, 1.0, 1.0, 0.0, 0.0], [u - c * nx, u, u + c * nx, lx, mx], [v - c * ny, v, v + c * ny, ly, my],
                 [w - c * nz, w, w + c * nz, lz, mz], [H - qn * c, q2, H + qn * c, ql, qm]]

            def char(n, pts):
                return [sum(L[n][m] * pt[m] for m in range(5)) for pt in pts]
            f7 = [(_weno7(char(n, P7), s0) + _weno7(char(n, M7), s0)) / 12.0 for n in range(5)]
            f5 = [(_weno5(char(n, P7[1:6]), s0) + _weno5(char(n, M7[1:6]), s0)) / 6.0 for n in range(5)]
            w7 = np.stack([sum(f7[k] * R[n][k] for k in range(5)) for n in range(5)])
            w5 = np.stack([sum(f5[k] * R[n][k] for k in range(5)) for n in range(5)])
        out.append(np.where(br == 0, up7, np.where(br == 1, w7, np.where(br == 2, w5, nnd))))
    F = np.stack(out, axis=1)  # (5, faces along d, t1, t2) with d-first order
    return np.moveaxis(F, 1, 3 - d)


def divergence(P, F, J, Fv=None):
    """dUdt at interior cells (U layout, ghosts zero): J (dF + CD4 dFv) (div.jl:1-50)."""
    out = np.zeros((5, P.nz + 8, P.ny + 8, P.nx + 8))
    Fx, Fy, Fz = F
    inv = (Fx[..., :-1] - Fx[..., 1:]) + (Fy[:, :, :-1] - Fy[:, :, 1:]) + (Fz[:, :-1] - Fz[:, 1:])
    I = (slice(NG, -NG),) * 3
    Jc = J[I]
    out[(slice(None),) + I] = inv * Jc
    if Fv is not None:
        for n in range(4):
            acc = 0.0
            for d, A in enumerate(Fv):
                a = _along(A[n], d)  # d-first, transverse full (N+4); cells c -> index c - 2
                tr = [slice(2, -2)] * 2
                ctr = a[(slice(2, -2), *tr)]
                m2, m1 = a[(slice(0, -4), *tr)], a[(slice(1, -3), *tr)]
                p1, p2 = a[(slice(3, -1), *tr)], a[(slice(4, None), *tr)]
                dv = (1 / 12) * (m2 - p2) + (-2 / 3) * (m1 - p1)
                acc = acc + np.moveaxis(dv[None], 1, 3 - d)[0]
                del ctr
            out[(n + 1,) + I] += acc * Jc
    return out


def _dcoord(f, axis):
    """CD6 in the interior, one-sided CD2 in the three outer layers (parse_mesh.jl:139-235)."""
    g = np.moveaxis(f, axis, 0)
    n = g.shape[0]
    d = np.empty_like(g)
    d[3:n - 3] = (1 / 60) * (g[6:] - g[:n - 6]) - (3 / 20) * (g[5:n - 1] - g[1:n - 5]) + (3 / 4) * (g[4:n - 2] - g[2:n - 4])
    for i in range(3):
        d[i] = 2 * g[i + 1] - 0.5 * g[i + 2] - 1.5 * g[i]
        j = n - 1 - i
        d[j] = -2 * g[j - 1] + 0.5 * g[j - 2] + 1.5 * g[j]
    return np.moveaxis(d, 0, axis)


def metrics(x, y, z):
    """(nine J^-1-scaled metrics in metrics.h5 order, J) from coordinates (parse_mesh.jl)."""
    xxi, yxi, zxi = (_dcoord(a, 2) for a in (x, y, z))
    xet, yet, zet = (_dcoord(a, 1) for a in (x, y, z))
    xze, yze, zze = (_dcoord(a, 0) for a in (x, y, z))
    J = 1 / (xxi * (yet * zze - yze * zet) - xet * (yxi * zze - yze * zxi) + xze * (yxi * zet - yet * zxi))
    m = [yet * zze - yze * zet, xze * zet - xet * zze, xet * yze - xze * yet,
         yze * zxi - yxi * zze, xxi * zze - xze * zxi, xze * yxi - xxi * yze,
         yxi * zet - yet * zxi, xet * zxi - xxi * zet, xxi * yet - xet * yxi]
    return m, J


def rhs(P, Q, x, y, z):
    """Inviscid RHS at interior cells from a ghost-filled Q and coordinates."""
    m, J = metrics(x, y, z)
    phi = sensor(Q)
    F = []
    for d in range(3):
        A = m[3 * d:3 * d + 3]
        S = np.sqrt(A[0] ** 2 + A[1] ** 2 + A[2] ** 2)
        Fp, Fm = split(P, Q, *A, S)
        F.append(face_flux(P, d, phi, S, Fp, Fm, Q, *A))
    return divergence(P, F, J)
