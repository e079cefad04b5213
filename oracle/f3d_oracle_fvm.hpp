// f3d_oracle_fvm.hpp — CPU restatement of the reference's finite-volume RHS (FVM.jl).
//
// TEST INFRASTRUCTURE ONLY (the oracle): included by oracle_capi.cpp.
//
// Per face of direction d (faces between cells i and i+1, 1-based, i = NG..N+NG):
//   geometry (FVM.jl:16-29 / 251-264 / 466-479): two face diagonals from corner points that
//     average eight cell centres, n = +-0.5 d1 x d2, Area = sqrt(|n|^2 + 1e-20), n /= Area;
//   sensor (FVM.jl:33): max of phi over cells i-2..i+3;
//   phi < phi1: the linear scheme on the conserved variables U (FVM.jl:42-60);
//   else, Eigen_reconstruct (FVM.jl:65-228): Roe averages of Q at i, i+1, tangent basis
//     (l, m), left eigenvectors L projecting U, WENO7 (phi < phi2, eps 1e-10), WENO5
//     (phi < phi3, eps 1e-8) or minmod on each characteristic field, right eigenvectors R
//     projecting back; or Conser_reconstruct (FVM.jl:739-855): the same schemes per
//     conserved component;
//   HLLC flux (FVM.jl:1224-1357) of (UL, UR) along n, times Area.
// Output: F in the shape of Fx/Fy/Fz ((Nx+1,Ny,Nz,5) for d = 0 ...), as FVM.jl:230-236.
#pragma once
#include "f3d_oracle.hpp"

namespace f3do {

// FVM.jl:1224-1357 HLLC_Flux: UL, UR conserved; n unit normal; writes the flux along n.
template <class R> void hllc_flux(const Consts<R>& C, const R UL[5], const R UR[5], R nx, R ny, R nz, R F[5]) {
    const R g = C.gamma;
    const R rL = UL[0], irL = R(1) / rL;
    const R uL = UL[1] * irL, vL = UL[2] * irL, wL = UL[3] * irL, EL = UL[4];
    const R pL = (g - R(1)) * (EL - R(0.5) * rL * (uL * uL + vL * vL + wL * wL));
    const R cL = sqrt(abs(g * pL * irL));
    const R qL = uL * nx + vL * ny + wL * nz;
    const R rR = UR[0], irR = R(1) / rR;
    const R uR = UR[1] * irR, vR = UR[2] * irR, wR = UR[3] * irR, ER = UR[4];
    const R pR = (g - R(1)) * (ER - R(0.5) * rR * (uR * uR + vR * vR + wR * wR));
    const R cR = sqrt(abs(g * pR * irR));
    const R qR = uR * nx + vR * ny + wR * nz;
    // Roe averages (FVM.jl:1256-1275)
    const R sL = sqrt(rL), sR = sqrt(rR), isum = R(1) / (sL + sR);
    const R ur = (sL * uL + sR * uR) * isum, vr = (sL * vL + sR * vR) * isum, wr = (sL * wL + sR * wR) * isum;
    const R qr = ur * nx + vr * ny + wr * nz;
    const R HL = (EL + pL) * irL, HR = (ER + pR) * irR;
    const R Hr = (sL * HL + sR * HR) * isum;
    const R v2r = ur * ur + vr * vr + wr * wr;
    const R cr = sqrt(abs((g - R(1)) * (Hr - R(0.5) * v2r)));
    const R SL = jmin(qL - cL, qr - cr);
    const R SR = jmax(qR + cR, qr + cr);
    const R Ss = (pR - pL + rL * qL * (SL - qL) - rR * qR * (SR - qR)) /
                 (rL * (SL - qL) - rR * (SR - qR) + R(1e-12));
    auto phys = [&](R r, R u, R v, R w, R E, R p, R q, R out[5]) {
        out[0] = r * q;
        out[1] = r * u * q + p * nx;
        out[2] = r * v * q + p * ny;
        out[3] = r * w * q + p * nz;
        out[4] = (E + p) * q;
    };
    if (SL >= R(0)) {
        phys(rL, uL, vL, wL, EL, pL, qL, F);
    } else if (SR <= R(0)) {
        phys(rR, uR, vR, wR, ER, pR, qR, F);
    } else if (Ss >= R(0)) {  // left star state (SL < 0 here)
        R FL[5];
        phys(rL, uL, vL, wL, EL, pL, qL, FL);
        const R f = rL * (SL - qL) / (SL - Ss);
        const R Us[5] = {f, f * (uL + (Ss - qL) * nx), f * (vL + (Ss - qL) * ny), f * (wL + (Ss - qL) * nz),
                         f * (EL * irL + (Ss - qL) * (Ss + pL / (rL * (SL - qL))))};
        for (int n = 0; n < 5; n++) F[n] = FL[n] + SL * (Us[n] - UL[n]);
    } else {  // right star state
        R FR[5];
        phys(rR, uR, vR, wR, ER, pR, qR, FR);
        const R f = rR * (SR - qR) / (SR - Ss);
        const R Us[5] = {f, f * (uR + (Ss - qR) * nx), f * (vR + (Ss - qR) * ny), f * (wR + (Ss - qR) * nz),
                         f * (ER * irR + (Ss - qR) * (Ss + pR / (rR * (SR - qR))))};
        for (int n = 0; n < 5; n++) F[n] = FR[n] + SR * (Us[n] - UR[n]);
    }
}

// WENO7 of FVM.jl:124-141 (eps 1e-10): V1..V7 in upwind order, returns the value.
template <class R> inline R fvm_weno7(const R V[7], R ss) {
    const R V1 = V[0], V2 = V[1], V3 = V[2], V4 = V[3], V5 = V[4], V6 = V[5], V7 = V[6];
    const R q1 = R(-3) * V1 + R(13) * V2 - R(23) * V3 + R(25) * V4;
    const R q2 = V2 - R(5) * V3 + R(13) * V4 + R(3) * V5;
    const R q3 = -V3 + R(7) * V4 + R(7) * V5 - V6;
    const R q4 = R(3) * V4 + R(13) * V5 - R(5) * V6 + V7;
    const R I1 = V1 * (R(547) * V1 - R(3882) * V2 + R(4642) * V3 - R(1854) * V4) +
                 V2 * (R(7043) * V2 - R(17246) * V3 + R(7042) * V4) + V3 * (R(11003) * V3 - R(9402) * V4) +
                 V4 * (R(2107) * V4);
    const R I2 = V2 * (R(267) * V2 - R(1642) * V3 + R(1602) * V4 - R(494) * V5) +
                 V3 * (R(2843) * V3 - R(5966) * V4 + R(1922) * V5) + V4 * (R(3443) * V4 - R(2522) * V5) +
                 V5 * (R(547) * V5);
    const R I3 = V3 * (R(547) * V3 - R(2522) * V4 + R(1922) * V5 - R(494) * V6) +
                 V4 * (R(3443) * V4 - R(5966) * V5 + R(1602) * V6) + V5 * (R(2843) * V5 - R(1642) * V6) +
                 V6 * (R(267) * V6);
    const R I4 = V4 * (R(2107) * V4 - R(9402) * V5 + R(7042) * V6 - R(1854) * V7) +
                 V5 * (R(11003) * V5 - R(17246) * V6 + R(4642) * V7) + V6 * (R(7043) * V6 - R(3882) * V7) +
                 V7 * (R(547) * V7);
    const R e = R(1e-10);
    const R t1 = e + I1 * ss, t2 = e + I2 * ss, t3 = e + I3 * ss, t4 = e + I4 * ss;
    const R a1 = R(1) / (t1 * t1), a2 = R(12) / (t2 * t2), a3 = R(18) / (t3 * t3), a4 = R(4) / (t4 * t4);
    const R inv = R(1) / (a1 + a2 + a3 + a4);
    return inv * (a1 * q1 + a2 * q2 + a3 * q3 + a4 * q4) * (R(1) / R(12));
}

// WENO5 of FVM.jl:146-197 (eps 1e-8) on V2..V6 of the seven-point stencil.
template <class R> inline R fvm_weno5(const R V[7], R ss) {
    const R a = V[1], b = V[2], c = V[3], d = V[4], e5 = V[5];
    R t1 = a - R(2) * b + c, t2 = a - R(4) * b + R(3) * c;
    const R s1 = R(13) * t1 * t1 + R(3) * t2 * t2;
    t1 = b - R(2) * c + d;
    t2 = b - d;
    const R s2 = R(13) * t1 * t1 + R(3) * t2 * t2;
    t1 = c - R(2) * d + e5;
    t2 = R(3) * c - R(4) * d + e5;
    const R s3 = R(13) * t1 * t1 + R(3) * t2 * t2;
    const R e = R(1e-8);
    const R d1 = e + s1 * ss, d2 = e + s2 * ss, d3 = e + s3 * ss;
    const R a1 = R(1) / (d1 * d1), a2 = R(6) / (d2 * d2), a3 = R(3) / (d3 * d3);
    const R inv = R(1) / (a1 + a2 + a3);
    const R v1 = R(2) * a - R(7) * b + R(11) * c;
    const R v2 = -b + R(5) * c + R(2) * d;
    const R v3 = R(2) * c + R(5) * d - e5;
    return inv * (a1 * v1 + a2 * v2 + a3 * v3) * (R(1) / R(6));
}

// One side's value of the non-linear schemes on a seven-point stencil (upwind order):
// br 1 = WENO7, 2 = WENO5, 3 = minmod. The two sides' minmod forms differ as written in
// FVM.jl:204-205: left V4 + 0.5 minmod(V4 - V3, V5 - V4), right V4 - 0.5 minmod(V4 - V3,
// V4 - V5).
template <class R> inline R fvm_side(int br, bool right, const R V[7], R ss) {
    if (br == 1) return fvm_weno7(V, ss);
    if (br == 2) return fvm_weno5(V, ss);
    if (right) return V[3] - R(0.5) * minmod(V[3] - V[2], V[3] - V[4]);
    return V[3] + R(0.5) * minmod(V[3] - V[2], V[4] - V[3]);
}

// Face geometry of direction d at the face between cells (i,j,k) and (i,j,k)+e_d,
// 1-based full indices, from cell-centre coordinates (FVM.jl:16-29 and the j, k kernels).
template <class R>
void fvm_face_geometry(int d, const V4<const R>& X, const V4<const R>& Y, const V4<const R>& Z, long i, long j,
                       long k, R& nx, R& ny, R& nz, R& area) {
    // e_d and the two transverse directions a, b (in the kernels' order)
    long di[3] = {0, 0, 0}, da[3] = {0, 0, 0}, db[3] = {0, 0, 0};
    di[d] = 1;
    const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
    da[a] = 1;
    db[b] = 1;
    // the cell at (pa a + pb b) from the face's left cell (side 0) or right cell (side 1)
    auto at = [&](const V4<const R>& A, int pa, int pb, int side) -> R {
        return A(i + side * di[0] + pa * da[0] + pb * db[0], j + side * di[1] + pa * da[1] + pb * db[1],
                 k + side * di[2] + pa * da[2] + pb * db[2]);
    };
    // d1 = P(+a,+b) - P(-a,-b), d2 = P(-a,+b) - P(+a,-b), each corner the mean of 8 cells: the
    // twelve centres summed left to right in the kernels' order (FVM.jl:16-21, 251-256,
    // 466-471): (sa,0), (0,sb), (sa,sb), each on both sides, then (-sa,0), (0,-sb), (-sa,-sb)
    // subtracted
    auto diag = [&](const V4<const R>& A, int sa, int sb) {
        R s = at(A, sa, 0, 0);
        s += at(A, sa, 0, 1);
        s += at(A, 0, sb, 0);
        s += at(A, 0, sb, 1);
        s += at(A, sa, sb, 0);
        s += at(A, sa, sb, 1);
        s -= at(A, -sa, 0, 0);
        s -= at(A, -sa, 0, 1);
        s -= at(A, 0, -sb, 0);
        s -= at(A, 0, -sb, 1);
        s -= at(A, -sa, -sb, 0);
        s -= at(A, -sa, -sb, 1);
        return R(0.125) * s;
    };
    const R dx1 = diag(X, 1, 1), dy1 = diag(Y, 1, 1), dz1 = diag(Z, 1, 1);
    const R dx2 = diag(X, -1, 1), dy2 = diag(Y, -1, 1), dz2 = diag(Z, -1, 1);
    const R sgn = d == 1 ? R(-1) : R(1);  // (a, b) = (x, z) on j faces: x cross z = -y
    nx = sgn * R(0.5) * (dy1 * dz2 - dz1 * dy2);
    ny = sgn * R(0.5) * (dz1 * dx2 - dx1 * dz2);
    nz = sgn * R(0.5) * (dx1 * dy2 - dy1 * dx2);
    area = sqrt(nx * nx + ny * ny + nz * nz + R(1e-20));
    nx = nx / area;
    ny = ny / area;
    nz = nz / area;
}

// G: the type the face geometry is computed in (R by default; double with R = long double
// gives the extended-precision yardstick the FP64 normals, and so the same side of every
// |nz| = |ny| tie of the characteristic tangent basis).
template <class R, class G = R>
void fvm_face_flux(const f3d_params& P, int d, bool eigen, const R* phip, const R* Sp, const R* Qp, const R* Up,
                   const G* xp, const G* yp, const G* zp, R* Fp_out, int8_t* branch_out) {
    Grid g(P);
    Consts<R> C(P);
    const long NG = g.ng;
    const size_t nc = g.ncell();
    const long st = g.stride(d);
    const long fx = g.nx + (d == 0), fy = g.ny + (d == 1), fz = g.nz + (d == 2);
    const size_t nf = (size_t)fx * fy * fz;
    V4<const G> X{xp, g.nxt, g.nyt, g.nzt}, Y{yp, g.nxt, g.nyt, g.nzt}, Z{zp, g.nxt, g.nyt, g.nzt};
    const R gm = C.gamma - R(1);
#pragma omp parallel for schedule(static)
    for (long kf = 1; kf <= fz; kf++)
        for (long jf = 1; jf <= fy; jf++)
            for (long ifc = 1; ifc <= fx; ifc++) {
                // left cell of the face, 1-based full index (the kernels' i, j, k)
                const long i = ifc + NG - (d == 0), j = jf + NG - (d == 1), k = kf + NG - (d == 2);
                const long cL = (i - 1) + g.nxt * ((j - 1) + g.nyt * (k - 1));
                auto at = [&](const R* a, long off, int n) -> R { return a[cL + off * st + (size_t)n * nc]; };
                const size_t fo = (ifc - 1) + fx * ((jf - 1) + fy * (kf - 1));
                G gnx, gny, gnz, garea;
                fvm_face_geometry<G>(d, X, Y, Z, i, j, k, gnx, gny, gnz, garea);
                const R nx = R(gnx), ny = R(gny), nz = R(gnz), area = R(garea);
                R phimax = at(phip, -2, 0);
                for (long o = -1; o <= 3; o++) phimax = jmax(phimax, at(phip, o, 0));
                const int br = face_branch(C, phimax);
                if (branch_out) branch_out[fo] = (int8_t)br;
                R UL[5] = {R(0), R(0), R(0), R(0), R(0)}, UR[5] = {R(0), R(0), R(0), R(0), R(0)};
                if (br == 0) {  // FVM.jl:42-60: U[i-3..i+3] and U[i+4..i-2]
                    for (int n = 0; n < 5; n++) {
                        R VL[7], VR[7];
                        for (int m = 0; m < 7; m++) {
                            VL[m] = at(Up, m - 3, n);
                            VR[m] = at(Up, 4 - m, n);
                        }
                        UL[n] = linear7(C.lin, VL);
                        UR[n] = linear7(C.lin, VR);
                    }
                } else {
                    const R ss = R(2) / (at(Sp, 1, 0) + at(Sp, 0, 0));
                    if (!eigen) {  // Conser_reconstruct, FVM.jl:739-855
                        for (int n = 0; n < 5; n++) {
                            R VL[7], VR[7];
                            for (int m = 0; m < 7; m++) {
                                VL[m] = at(Up, m - 3, n);
                                VR[m] = at(Up, 4 - m, n);
                            }
                            UL[n] = fvm_side(br, false, VL, ss);
                            UR[n] = fvm_side(br, true, VR, ss);
                        }
                    } else {  // Eigen_reconstruct, FVM.jl:65-228
                        const R rl = at(Qp, 0, 0), rr = at(Qp, 1, 0);
                        const R srl = sqrt(rl), srr = sqrt(rr);
                        const R u = (srl * at(Qp, 0, 1) + srr * at(Qp, 1, 1)) / (srl + srr);
                        const R v = (srl * at(Qp, 0, 2) + srr * at(Qp, 1, 2)) / (srl + srr);
                        const R w = (srl * at(Qp, 0, 3) + srr * at(Qp, 1, 3)) / (srl + srr);
                        const R HLc = C.gamma / gm * at(Qp, 0, 4) / rl +
                                      R(0.5) * (sq(at(Qp, 0, 1)) + sq(at(Qp, 0, 2)) + sq(at(Qp, 0, 3)));
                        const R HRc = C.gamma / gm * at(Qp, 1, 4) / rr +
                                      R(0.5) * (sq(at(Qp, 1, 1)) + sq(at(Qp, 1, 2)) + sq(at(Qp, 1, 3)));
                        const R H = (srl * HLc + srr * HRc) / (srl + srr);
                        const R v2 = R(0.5) * (u * u + v * v + w * w);
                        const R c = sqrt(gm * (H - v2));
                        R lx, ly, lz;
                        if (abs(nz) <= abs(ny)) {
                            const R den = sqrt(nx * nx + ny * ny + R(1e-12));
                            lx = -ny / den; ly = nx / den; lz = R(0);
                        } else {
                            const R den = sqrt(nx * nx + nz * nz + R(1e-12));
                            lx = -nz / den; ly = R(0); lz = nx / den;
                        }
                        const R mx = ny * lz - nz * ly, my = nz * lx - nx * lz, mz = nx * ly - ny * lx;
                        const R invc = R(1) / c, invc2 = invc * invc;
                        const R Ku = gm * u * invc2, Kv = gm * v * invc2, Kw = gm * w * invc2;
                        const R Kv2 = gm * v2 * invc2, Kc2 = gm * invc2;
                        const R un = u * nx + v * ny + w * nz, ul = u * lx + v * ly + w * lz, um = u * mx + v * my + w * mz;
                        const R uni = un * invc, nxi = nx * invc, nyi = ny * invc, nzi = nz * invc;
                        const R h = R(0.5), mh = R(-0.5);
                        const R Lm[5][5] = {{h * (Kv2 + uni), mh * (Ku + nxi), mh * (Kv + nyi), mh * (Kw + nzi), h * Kc2},
                                            {R(1) - Kv2, Ku, Kv, Kw, -Kc2},
                                            {h * (Kv2 - uni), mh * (Ku - nxi), mh * (Kv - nyi), mh * (Kw - nzi), h * Kc2},
                                            {-ul, lx, ly, lz, R(0)},
                                            {-um, mx, my, mz, R(0)}};
                        const R Rm[5][5] = {{R(1), u - nx * c, v - ny * c, w - nz * c, H - un * c},
                                            {R(1), u, v, w, v2},
                                            {R(1), u + nx * c, v + ny * c, w + nz * c, H + un * c},
                                            {R(0), lx, ly, lz, ul},
                                            {R(0), mx, my, mz, um}};
                        for (int n = 0; n < 5; n++) {
                            R VL[7], VR[7];
                            for (int m = 0; m < 7; m++) {
                                const long oL = m - 3, oR = 4 - m;
                                VL[m] = Lm[n][0] * at(Up, oL, 0) + Lm[n][1] * at(Up, oL, 1) + Lm[n][2] * at(Up, oL, 2) +
                                        Lm[n][3] * at(Up, oL, 3) + Lm[n][4] * at(Up, oL, 4);
                                VR[m] = Lm[n][0] * at(Up, oR, 0) + Lm[n][1] * at(Up, oR, 1) + Lm[n][2] * at(Up, oR, 2) +
                                        Lm[n][3] * at(Up, oR, 3) + Lm[n][4] * at(Up, oR, 4);
                            }
                            const R vL = fvm_side(br, false, VL, ss), vR = fvm_side(br, true, VR, ss);
                            for (int q = 0; q < 5; q++) {
                                UL[q] += Rm[n][q] * vL;
                                UR[q] += Rm[n][q] * vR;
                            }
                        }
                    }
                }
                R Ff[5];
                hllc_flux<R>(C, UL, UR, nx, ny, nz, Ff);
                for (int n = 0; n < 5; n++) Fp_out[fo + n * nf] = Ff[n] * area;
            }
}

}  // namespace f3do
