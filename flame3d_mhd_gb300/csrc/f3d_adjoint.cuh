// f3d_adjoint.cuh — reverse-mode (vector-Jacobian) kernels of the FP64 RHS pieces.
//
// Each function takes the forward inputs and the cotangent of the outputs and returns (or
// accumulates) the cotangent of the inputs. Branches (sign splits, minmod, the hybrid
// scheme choice, the c2Prim clamps) are frozen at the forward value: the result is the
// exact derivative of the branch taken, which is the discrete adjoint of the scheme.
#pragma once
#include "f3d_common.cuh"
#include "f3d_flux.cuh"

namespace f3d {

// ---- c2Prim (utils.jl:2-30): q = (rho,u,v,w,p,T) from U; qb -> Ub ----------------------
__device__ __forceinline__ void c2prim_vjp(const DevParams& P, const double U[5], const double qb[6], double Ub[5]) {
    const bool rho_free = U[0] > P.eps_clamp;
    const double rho = rho_free ? U[0] : P.eps_clamp;
    const double rinv = 1.0 / rho;
    const double u = U[1] * rinv, v = U[2] * rinv, w = U[3] * rinv;
    const double ke = u * u + v * v + w * w;
    const double eraw = U[4] - 0.5 * rho * ke;
    const bool e_free = eraw > P.eps_clamp;
    const double ei = e_free ? eraw : P.eps_clamp;
    const double p = P.gm1 * ei;
    const double Tr = qb[5] * rinv * P.inv_rg;  // T = p/(rho Rg)
    double pb = qb[4] + Tr;
    double rhob = qb[0] - Tr * p * rinv;
    const double eb = e_free ? P.gm1 * pb : 0.0;
    Ub[4] = eb;
    rhob += -0.5 * ke * eb;
    const double keb = -0.5 * rho * eb;
    const double ub = qb[1] + 2.0 * u * keb, vb = qb[2] + 2.0 * v * keb, wb = qb[3] + 2.0 * w * keb;
    Ub[1] = ub * rinv;
    Ub[2] = vb * rinv;
    Ub[3] = wb * rinv;
    const double rinvb = ub * U[1] + vb * U[2] + wb * U[3];
    rhob += -rinvb * rinv * rinv;
    Ub[0] = rho_free ? rhob : 0.0;
}

// ---- flux splitting (split.jl) -------------------------------------------------------
// q = (rho,u,v,w,p,T); c = the split's sound speed; fpb/fmb cotangents of Fp/Fm.
// Accumulates into qb[6] (the sound-speed dependence goes to T for SW, to p and rho for LF).
// mg (optional): cotangents of the metric inputs, {A1, A2, A3, H1, H2, H3, |A|} += .
// Steger-Warming: the reverse of split_cell's FP64 form (the same function of q, c and the
// metric row as split.jl:2-68): E1 = |A| (Ah.u), the eigenvalues scaled by t1 = rho/(2 gamma)
// and routed by their sign pattern, the eigenvectors' velocities u -+ c Ah and enthalpies
// H -+ c Un. The metric enters only through Ah and |A| (A's own cotangent stays 0; the caller
// folds Ah and |A| back onto A).
__device__ __forceinline__ void split_sw_vjp(const Cst<double>& K, const double q[6], double c, double A1, double A2,
                                             double A3, double H1, double H2, double H3, double ss,
                                             const double fpb[5], const double fmb[5], double qb[6],
                                             double* mg = nullptr) {
    (void)A1; (void)A2; (void)A3;
    const double rho = q[0], u = q[1], v = q[2], w = q[3];
    const double tss = (rho * ss) * K.inv_2g;
    const double Un = H1 * u + H2 * v + H3 * w;
    const double e1 = tss * Un, tcs = tss * c;
    const double e2 = e1 - tcs, e3 = e1 + tcs;
    const double q2 = u * u + v * v + w * w;
    const double vv = K.gm1 * q2;
    const double Hh = 0.5 * q2 + (K.inv_gm1 * c) * c;
    const double cUn = c * Un;
    const bool e2pos = __double2hiint(e2) >= 0, e3pos = __double2hiint(e3) >= 0;
    double ub = 0, vb = 0, wb = 0, cb = 0, Hb1 = 0, Hb2 = 0, Hb3 = 0, vvb = 0, Hhb = 0, cUnb = 0;
    double e1b, e2b, e3b;
    if (e2pos || !e3pos) {  // f = a1 + e2 + e3, (a1 + e2 + e3) u + c (e3 - e2) Ah, e1 vv + (e2 + e3) H + (e3 - e2) c Un
        const double* g = e2pos ? fpb : fmb;
        const double a1 = K.two_gm1 * e1, s23 = e2 + e3, d23 = e3 - e2;
        const double f0 = a1 + s23, dc = d23 * c;
        const double f0b = g[0] + g[1] * u + g[2] * v + g[3] * w;
        const double dcb = g[1] * H1 + g[2] * H2 + g[3] * H3;
        ub += g[1] * f0; vb += g[2] * f0; wb += g[3] * f0;
        Hb1 += g[1] * dc; Hb2 += g[2] * dc; Hb3 += g[3] * dc;
        vvb += g[4] * e1;
        Hhb += g[4] * s23;
        cUnb += g[4] * d23;
        cb += dcb * d23;
        const double s23b = g[4] * Hh + f0b, d23b = g[4] * cUn + dcb * c;
        e1b = g[4] * vv + K.two_gm1 * f0b;
        e2b = s23b - d23b;
        e3b = s23b + d23b;
    } else {  // e2 < 0 <= e3: Fp from e3 (and e1 >= 0), Fm from e2 (and e1 < 0)
        const bool e1pos = __double2hiint(e1) >= 0;
        const double e1p = e1pos ? e1 : 0.0, e1m = e1pos ? 0.0 : e1;
        const double fp0 = K.two_gm1 * e1p + e3, e3c = e3 * c;
        const double fm0 = K.two_gm1 * e1m + e2, e2c = e2 * c;
        const double* g = fpb;
        const double* h = fmb;
        const double fp0b = g[0] + g[1] * u + g[2] * v + g[3] * w;
        const double fm0b = h[0] + h[1] * u + h[2] * v + h[3] * w;
        const double e3cb = g[1] * H1 + g[2] * H2 + g[3] * H3;
        const double e2cb = -(h[1] * H1 + h[2] * H2 + h[3] * H3);
        ub += g[1] * fp0 + h[1] * fm0;
        vb += g[2] * fp0 + h[2] * fm0;
        wb += g[3] * fp0 + h[3] * fm0;
        Hb1 += g[1] * e3c - h[1] * e2c;
        Hb2 += g[2] * e3c - h[2] * e2c;
        Hb3 += g[3] * e3c - h[3] * e2c;
        vvb += g[4] * e1p + h[4] * e1m;
        Hhb += g[4] * e3 + h[4] * e2;
        cUnb += g[4] * e3 - h[4] * e2;
        cb += e3cb * e3 + e2cb * e2;
        e3b = fp0b + e3cb * c + g[4] * (Hh + cUn);
        e2b = fm0b + e2cb * c + h[4] * (Hh - cUn);
        // e1+ = max(e1, 0), e1- = min(e1, 0): the cotangent of the side e1 lies on
        e1b = e1pos ? g[4] * vv + K.two_gm1 * fp0b : h[4] * vv + K.two_gm1 * fm0b;
    }
    // e2 = e1 - tcs, e3 = e1 + tcs; e1 = tss Un, tcs = tss c; cUn = c Un
    e1b += e2b + e3b;
    const double tcsb = e3b - e2b;
    const double tssb = e1b * Un + tcsb * c;
    const double Unb = e1b * tss + cUnb * c;
    cb += tcsb * tss + cUnb * Un;
    // Hh = q2/2 + c^2/(gamma-1), vv = (gamma-1) q2, q2 = |u|^2, Un = Ah.u
    const double q2b = 0.5 * Hhb + K.gm1 * vvb;
    cb += 2.0 * (K.inv_gm1 * c) * Hhb;
    ub += 2.0 * u * q2b + H1 * Unb;
    vb += 2.0 * v * q2b + H2 * Unb;
    wb += 2.0 * w * q2b + H3 * Unb;
    if (mg) {
        mg[3] += Hb1 + u * Unb;
        mg[4] += Hb2 + v * Unb;
        mg[5] += Hb3 + w * Unb;
        mg[6] += tssb * rho * K.inv_2g;
    }
    qb[0] += tssb * ss * K.inv_2g;
    qb[1] += ub;
    qb[2] += vb;
    qb[3] += wb;
    // c = sqrt(gamma Rg T)
    qb[5] += cb * K.grg / (2.0 * c);
}

__device__ __forceinline__ void split_lf_vjp(const Cst<double>& K, const double q[6], double c, double A1, double A2,
                                             double A3, double ss, const double fpb[5], const double fmb[5],
                                             double qb[6], double* mg = nullptr) {
    const double rho = q[0], u = q[1], v = q[2], w = q[3], p = q[4];
    const double un = A1 * u + A2 * v + A3 * w;
    const double l0 = fabs(un) + c * ss;
    const double kin = u * u + v * v + w * w;
    const double E0 = p * K.inv_gm1 + 0.5 * rho * kin;
    const double Uc[5] = {rho, rho * u, rho * v, rho * w, E0};
    double Fb[5], Ucb[5], l0b = 0;
    for (int n = 0; n < 5; n++) {
        Fb[n] = 0.5 * (fpb[n] + fmb[n]);
        const double d = 0.5 * (fpb[n] - fmb[n]);
        l0b += d * Uc[n];
        Ucb[n] = l0 * d;
    }
    // F = (rho un, rho u un + A1 p, rho v un + A2 p, rho w un + A3 p, (E0 + p) un)
    double rhob = Fb[0] * un + Ucb[0], ub = 0, vb = 0, wb = 0, pb = 0, E0b = Ucb[4];
    double unb = Fb[0] * rho + Fb[1] * rho * u + Fb[2] * rho * v + Fb[3] * rho * w + Fb[4] * (E0 + p);
    rhob += Fb[1] * u * un + Fb[2] * v * un + Fb[3] * w * un;
    ub += Fb[1] * rho * un;
    vb += Fb[2] * rho * un;
    wb += Fb[3] * rho * un;
    pb += A1 * Fb[1] + A2 * Fb[2] + A3 * Fb[3] + Fb[4] * un;
    E0b += Fb[4] * un;
    // Uc momentum components
    rhob += Ucb[1] * u + Ucb[2] * v + Ucb[3] * w;
    ub += Ucb[1] * rho;
    vb += Ucb[2] * rho;
    wb += Ucb[3] * rho;
    // E0 = p/(g-1) + rho kin / 2
    pb += E0b * K.inv_gm1;
    rhob += E0b * 0.5 * kin;
    ub += E0b * rho * u;
    vb += E0b * rho * v;
    wb += E0b * rho * w;
    // l0 = |un| + c ss
    unb += l0b * (un >= 0.0 ? 1.0 : -1.0);
    const double cb = l0b * ss;
    if (mg) {  // un = A . u; the pressure terms A_k p; l0 = |un| + c ss (no A/|A| here)
        mg[0] += unb * u + Fb[1] * p;
        mg[1] += unb * v + Fb[2] * p;
        mg[2] += unb * w + Fb[3] * p;
        mg[6] += l0b * c;
    }
    ub += A1 * unb;
    vb += A2 * unb;
    wb += A3 * unb;
    // c = sqrt(gamma p / rho)
    pb += cb * K.gamma / (2.0 * c * rho);
    rhob += -cb * c / (2.0 * rho);
    qb[0] += rhob;
    qb[1] += ub;
    qb[2] += vb;
    qb[3] += wb;
    qb[4] += pb;
}

// van Leer (split.jl:110-183) and AUSM (split.jl:185-255): Mach-number splits with
// c = sqrt(gamma p / rho) (the precomputed sound speed of those splits). The branch |M| >= 1
// (all flux to one side) is frozen at the forward value, as every other switch.
// mg (optional): cotangents {A1, A2, A3, -, -, -, |A|} +=.
__device__ __forceinline__ void split_mach_vjp(int method, const Cst<double>& K, const double q[6], double c, double A1,
                                               double A2, double A3, double ss, const double fpb[5],
                                               const double fmb[5], double qb[6], double* mg = nullptr) {
    const double rho = q[0], u = q[1], v = q[2], w = q[3], p = q[4];
    const double g = K.gamma;
    const bool vl = method == F3D_SPLIT_VL;
    const double un = A1 * u + A2 * v + A3 * w;
    const double M = un / (c * ss);  // the forward's expression, so the branch below is its branch
    const double kin = u * u + v * v + w * w;
    double rhob = 0, ub = 0, vb = 0, wb = 0, pb = 0, cb = 0, unb = 0, Mb = 0, kinb = 0, ssb = 0;
    double Ab[3] = {0, 0, 0};
    if (M <= -1.0 || M >= 1.0) {
        const double* gb = M <= -1.0 ? fmb : fpb;  // the side that carries the whole flux
        // full = (rho un, rho u un + A1 p, rho v un + A2 p, rho w un + A3 p, f4)
        rhob += gb[0] * un + (gb[1] * u + gb[2] * v + gb[3] * w) * un;
        unb += rho * (gb[0] + gb[1] * u + gb[2] * v + gb[3] * w);
        ub += gb[1] * rho * un;
        vb += gb[2] * rho * un;
        wb += gb[3] * rho * un;
        pb += A1 * gb[1] + A2 * gb[2] + A3 * gb[3];
        Ab[0] += gb[1] * p;
        Ab[1] += gb[2] * p;
        Ab[2] += gb[3] * p;
        if (vl) {  // f4 = (E0 + p) un, E0 = p/(g-1) + rho kin/2
            const double E0 = p * K.inv_gm1 + 0.5 * rho * kin;
            const double E0b = gb[4] * un;
            pb += gb[4] * un + E0b * K.inv_gm1;
            unb += gb[4] * (E0 + p);
            rhob += E0b * 0.5 * kin;
            kinb += E0b * 0.5 * rho;
        } else {  // f4 = rho h un, h = g p / (rho (g-1)) + kin/2
            const double h = g * p / (rho * K.gm1) + 0.5 * kin;
            const double hb = gb[4] * rho * un;
            rhob += gb[4] * h * un - hb * g * p / (rho * rho * K.gm1);
            unb += gb[4] * rho * h;
            pb += hb * g / (rho * K.gm1);
            kinb += 0.5 * hb;
        }
    } else if (vl) {
        const double unn = un / ss;
        const double Mp = M + 1.0, Mm = M - 1.0;
        const double f1p = rho * c * 0.25 * (Mp * Mp) * ss;
        const double f1m = -rho * c * 0.25 * (Mm * Mm) * ss;
        const double gs = g * ss;
        const double t1 = (-unn + 2.0 * c) / gs, t2 = (-unn - 2.0 * c) / gs;
        const double t3 = 1.0 / (2.0 * (g * g - 1.0));
        const double ep = K.gm1 * unn + 2.0 * c, em = K.gm1 * unn - 2.0 * c;
        const double t4 = 0.5 * (kin - unn * unn);
        const double Bp[5] = {1.0, A1 * t1 + u, A2 * t1 + v, A3 * t1 + w, ep * ep * t3 + t4};
        const double Bm[5] = {1.0, A1 * t2 + u, A2 * t2 + v, A3 * t2 + w, em * em * t3 + t4};
        double f1pb = 0, f1mb = 0;
        for (int n = 0; n < 5; n++) {
            f1pb += fpb[n] * Bp[n];
            f1mb += fmb[n] * Bm[n];
        }
        double t1b = 0, t2b = 0, t4b = 0, unnb = 0;
        const double Ap[3] = {A1, A2, A3};
        for (int j = 0; j < 3; j++) {
            const double bp = f1p * fpb[1 + j], bm = f1m * fmb[1 + j];
            t1b += Ap[j] * bp;
            t2b += Ap[j] * bm;
            Ab[j] += t1 * bp + t2 * bm;
        }
        ub += f1p * fpb[1] + f1m * fmb[1];
        vb += f1p * fpb[2] + f1m * fmb[2];
        wb += f1p * fpb[3] + f1m * fmb[3];
        const double E4p = f1p * fpb[4], E4m = f1m * fmb[4];
        const double epb = 2.0 * ep * t3 * E4p, emb = 2.0 * em * t3 * E4m;
        t4b += E4p + E4m;
        unnb += K.gm1 * (epb + emb);
        cb += 2.0 * (epb - emb);
        unnb -= (t1b + t2b) / gs;
        cb += 2.0 * (t1b - t2b) / gs;
        ssb -= (t1b * t1 + t2b * t2) / ss;
        kinb += 0.5 * t4b;
        unnb -= unn * t4b;
        // f1p = rho c (M+1)^2 ss / 4, f1m = -rho c (M-1)^2 ss / 4
        rhob += 0.25 * c * ss * (f1pb * Mp * Mp - f1mb * Mm * Mm);
        cb += 0.25 * rho * ss * (f1pb * Mp * Mp - f1mb * Mm * Mm);
        ssb += 0.25 * rho * c * (f1pb * Mp * Mp - f1mb * Mm * Mm);
        Mb += 0.5 * rho * c * ss * (f1pb * Mp - f1mb * Mm);
        unb += unnb / ss;
        ssb -= unnb * unn / ss;
    } else {  // AUSM, subsonic
        const double Mp = M + 1.0, Mm = M - 1.0;
        const double rcs = rho * c * ss;
        const double f_p = 0.25 * (Mp * Mp) * rcs, f_m = -0.25 * (Mm * Mm) * rcs;
        const double Pp = p * (0.25 * (Mp * Mp) * (2.0 - M)), Pm = p * (0.25 * (Mm * Mm) * (2.0 + M));
        const double h = g * p / (rho * K.gm1) + 0.5 * kin;
        const double f_pb = fpb[0] + fpb[1] * u + fpb[2] * v + fpb[3] * w + fpb[4] * h;
        const double f_mb = fmb[0] + fmb[1] * u + fmb[2] * v + fmb[3] * w + fmb[4] * h;
        const double Ppb = A1 * fpb[1] + A2 * fpb[2] + A3 * fpb[3];
        const double Pmb = A1 * fmb[1] + A2 * fmb[2] + A3 * fmb[3];
        Ab[0] += Pp * fpb[1] + Pm * fmb[1];
        Ab[1] += Pp * fpb[2] + Pm * fmb[2];
        Ab[2] += Pp * fpb[3] + Pm * fmb[3];
        ub += f_p * fpb[1] + f_m * fmb[1];
        vb += f_p * fpb[2] + f_m * fmb[2];
        wb += f_p * fpb[3] + f_m * fmb[3];
        const double hb = f_p * fpb[4] + f_m * fmb[4];
        // f_p, f_m
        const double rcsb = 0.25 * (f_pb * Mp * Mp - f_mb * Mm * Mm);
        Mb += 0.5 * rcs * (f_pb * Mp - f_mb * Mm);
        rhob += rcsb * c * ss;
        cb += rcsb * rho * ss;
        ssb += rcsb * rho * c;
        // Pp = p (M+1)^2 (2-M) / 4, Pm = p (M-1)^2 (2+M) / 4
        pb += Ppb * 0.25 * (Mp * Mp) * (2.0 - M) + Pmb * 0.25 * (Mm * Mm) * (2.0 + M);
        Mb += Ppb * p * 0.25 * (2.0 * Mp * (2.0 - M) - Mp * Mp) + Pmb * p * 0.25 * (2.0 * Mm * (2.0 + M) + Mm * Mm);
        // h = g p / (rho (g-1)) + kin / 2
        pb += hb * g / (rho * K.gm1);
        rhob -= hb * g * p / (rho * rho * K.gm1);
        kinb += 0.5 * hb;
    }
    // M = un / (c ss)
    const double cs = c * ss;
    unb += Mb / cs;
    cb -= Mb * M / c;
    ssb -= Mb * M / ss;
    ub += 2.0 * u * kinb;
    vb += 2.0 * v * kinb;
    wb += 2.0 * w * kinb;
    // un = A . (u, v, w)
    ub += A1 * unb;
    vb += A2 * unb;
    wb += A3 * unb;
    Ab[0] += u * unb;
    Ab[1] += v * unb;
    Ab[2] += w * unb;
    // c = sqrt(gamma p / rho)
    pb += cb * c / (2.0 * p);
    rhob -= cb * c / (2.0 * rho);
    if (mg) {
        mg[0] += Ab[0];
        mg[1] += Ab[1];
        mg[2] += Ab[2];
        mg[6] += ssb;
    }
    qb[0] += rhob;
    qb[1] += ub;
    qb[2] += vb;
    qb[3] += wb;
    qb[4] += pb;
}

// ---- WENO reconstructions: cotangents of the stencil values ---------------------------
// The reference normalises alpha_k = d_k / t_k^2, t_k = eps + IS_k s0, f = sum alpha q / sum alpha
// (schemes.jl:153-185, 233-252). With fb the cotangent of f (already divided by 12 or 6):
// qb_k = fb w_k, alphab_k = fb (q_k - f) / sum alpha, tb_k = -2 alpha_k / t_k alphab_k, and
// IS_k is a quadratic form whose gradient is formed from the coefficient table.
// s0b (optional): += the cotangent of the scale s0 (t_k = eps + IS_k s0).
__device__ __forceinline__ void weno5_vjp(const double V[5], double s0, double fb, double Vb[5],
                                          double* s0b = nullptr, double* fval = nullptr) {
    const double V1 = V[0], V2 = V[1], V3 = V[2], V4 = V[3], V5 = V[4];
    const double a1_ = V1 - 2 * V2 + V3, b1_ = V1 - 4 * V2 + 3 * V3;
    const double a2_ = V2 - 2 * V3 + V4, b2_ = V2 - V4;
    const double a3_ = V3 - 2 * V4 + V5, b3_ = 3 * V3 - 4 * V4 + V5;
    const double IS[3] = {13 * a1_ * a1_ + 3 * b1_ * b1_, 13 * a2_ * a2_ + 3 * b2_ * b2_, 13 * a3_ * a3_ + 3 * b3_ * b3_};
    const double d[3] = {1.0, 6.0, 3.0};
    const double q[3] = {2 * V1 - 7 * V2 + 11 * V3, -V2 + 5 * V3 + 2 * V4, 2 * V3 + 5 * V4 - V5};
    // two FP64 divisions: 1/t_k from 1/(t1 t2 t3), and 1/sum alpha
    const double t0 = 1e-16 + IS[0] * s0, t1 = 1e-16 + IS[1] * s0, t2 = 1e-16 + IS[2] * s0;
    const double t12 = t1 * t2, rall = 1.0 / (t0 * t12);
    const double it[3] = {t12 * rall, t0 * t2 * rall, t0 * t1 * rall};
    double al[3], sum = 0;
    for (int k = 0; k < 3; k++) {
        al[k] = d[k] * it[k] * it[k];
        sum += al[k];
    }
    const double rs = 1.0 / sum;
    double f = 0;
    for (int k = 0; k < 3; k++) f += al[k] * rs * q[k];
    if (fval) *fval = f;  // the forward value (6x the reconstruction)
    double qb[3], ISb[3];
    for (int k = 0; k < 3; k++) {
        const double wk = al[k] * rs;
        qb[k] = fb * wk;
        // alpha_k-bar = fb (q_k - f) / sum, t_k-bar = -2 alpha_k / t_k alpha_k-bar
        const double tb = -2.0 * fb * (q[k] - f) * wk * it[k];
        ISb[k] = s0 * tb;
        if (s0b) *s0b += IS[k] * tb;
    }
    for (int j = 0; j < 5; j++) Vb[j] = 0.0;
    // q
    Vb[0] += 2 * qb[0]; Vb[1] += -7 * qb[0]; Vb[2] += 11 * qb[0];
    Vb[1] += -qb[1]; Vb[2] += 5 * qb[1]; Vb[3] += 2 * qb[1];
    Vb[2] += 2 * qb[2]; Vb[3] += 5 * qb[2]; Vb[4] += -qb[2];
    // IS_k = 13 a^2 + 3 b^2
    double ga = 26 * a1_ * ISb[0], gb = 6 * b1_ * ISb[0];
    Vb[0] += ga + gb; Vb[1] += -2 * ga - 4 * gb; Vb[2] += ga + 3 * gb;
    ga = 26 * a2_ * ISb[1]; gb = 6 * b2_ * ISb[1];
    Vb[1] += ga + gb; Vb[2] += -2 * ga; Vb[3] += ga - gb;
    ga = 26 * a3_ * ISb[2]; gb = 6 * b3_ * ISb[2];
    Vb[2] += ga + 3 * gb; Vb[3] += -2 * ga - 4 * gb; Vb[4] += ga + gb;
}

// Upper-triangular coefficients of the WENO7 smoothness indicators (schemes.jl:160-175):
// IS_k = sum_{i<=j} C[k][i][j] V_{k+i} V_{k+j} over the 4 points of sub-stencil k.
__device__ __constant__ const double kW7IS[4][4][4] = {
    {{547, -3882, 4642, -1854}, {0, 7043, -17246, 7042}, {0, 0, 11003, -9402}, {0, 0, 0, 2107}},
    {{267, -1642, 1602, -494}, {0, 2843, -5966, 1922}, {0, 0, 3443, -2522}, {0, 0, 0, 547}},
    {{547, -2522, 1922, -494}, {0, 3443, -5966, 1602}, {0, 0, 2843, -1642}, {0, 0, 0, 267}},
    {{2107, -9402, 7042, -1854}, {0, 11003, -17246, 4642}, {0, 0, 7043, -3882}, {0, 0, 0, 547}}};
__device__ __constant__ const double kW7Q[4][4] = {{-3, 13, -23, 25}, {1, -5, 13, 3}, {-1, 7, 7, -1}, {3, 13, -5, 1}};

__device__ __forceinline__ void weno7_vjp(const double V[7], double s0, double fb, double Vb[7],
                                          double* s0b = nullptr, double* fval = nullptr) {
    // smoothness indicators in the difference form of weno7_is (f3d_flux.cuh):
    // IS_k = D1 y1^2 + D2 y2^2 + D3 d3^2, y1 = d1 + a d2 + b d3, y2 = d2 + c d3, d_j the first
    // differences of sub-stencil k; equal to the reference's quadratic form (schemes.jl:160-175)
    using C = W7Ldl<double>;
    const double dk[4] = {1.0, 12.0, 18.0, 4.0};
    double q[4], t[4], IS[4], y1[4], y2[4], d3[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        double qq = 0;
#pragma unroll
        for (int i = 0; i < 4; i++) qq += kW7Q[k][i] * V[k + i];
        q[k] = qq;
        const double e1 = V[k + 1] - V[k], e2 = V[k + 2] - V[k + 1], e3 = V[k + 3] - V[k + 2];
        y1[k] = e1 + C::a(k) * e2 + C::b(k) * e3;
        y2[k] = e2 + C::c(k) * e3;
        d3[k] = e3;
        IS[k] = C::D1(k) * (y1[k] * y1[k]) + C::D2(k) * (y2[k] * y2[k]) + C::D3(k) * (e3 * e3);
        t[k] = 1e-20 + IS[k] * s0;
    }
    // two FP64 divisions: 1/t_k from 1/(t1 t2 t3 t4), and 1/sum alpha
    const double t01 = t[0] * t[1], t23 = t[2] * t[3], rall = 1.0 / (t01 * t23);
    const double it[4] = {t[1] * t23 * rall, t[0] * t23 * rall, t01 * t[3] * rall, t01 * t[2] * rall};
    double al[4], sum = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        al[k] = dk[k] * it[k] * it[k];
        sum += al[k];
    }
    const double rs = 1.0 / sum;
    double f = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) f += al[k] * rs * q[k];
    if (fval) *fval = f;  // the forward value (12x the reconstruction)
#pragma unroll
    for (int j = 0; j < 7; j++) Vb[j] = 0.0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const double wk = al[k] * rs;
        const double qb = fb * wk;
        const double tb = -2.0 * fb * (q[k] - f) * wk * it[k];
        const double ISb = s0 * tb;
        if (s0b) *s0b += IS[k] * tb;
#pragma unroll
        for (int i = 0; i < 4; i++) Vb[k + i] += kW7Q[k][i] * qb;
        // IS_k through y1, y2, d3 back to the differences and the stencil values
        const double y1b = 2.0 * C::D1(k) * y1[k] * ISb, y2b = 2.0 * C::D2(k) * y2[k] * ISb;
        const double e3b = 2.0 * C::D3(k) * d3[k] * ISb + C::b(k) * y1b + C::c(k) * y2b;
        const double e2b = C::a(k) * y1b + y2b, e1b = y1b;
        Vb[k] -= e1b;
        Vb[k + 1] += e1b - e2b;
        Vb[k + 2] += e2b - e3b;
        Vb[k + 3] += e3b;
    }
}

// ---- characteristic-wise WENO7 / WENO5 face (schemes.jl:756-999) ---------------------
// Forward: face state (u, v, w, T) and metric row A = the arithmetic means at the two cells
// beside the face; n = A s0; tangent basis l (from n, switching on |nz| <= |ny|) and m = n x l;
// left eigenvectors L (rows) from (u, v, w, T, n, l, m); per characteristic field k the
// projected split fluxes L_k . Fp / L_k . Fm on the stencil, WENO of each side, their sum x
// 1/12 (WENO7) or 1/6 (WENO5); the face flux is R flux with the right eigenvectors R.
// Reverse for the face cotangent Fb: the split-flux cotangents are added through addP(n, pos,
// value) / addM(n, pos, value); stb[7] += cotangents of (u, v, w, T, A1, A2, A3) of the face
// state; *s0b += the cotangent of s0 (weights' scale and n = A s0) when s0b is set.
// br: 1 = WENO7, 2 = WENO5; t: the face's stencil origin (positions t..t+7).
template <bool W7, class FPA, class FMA, class ADDP, class ADDM>
__device__ __forceinline__ void char_face_vjp_t(int t, const DevParams& P, double s0, const double st[7],
                                                const double Fb[5], FPA FP, FMA FM, ADDP addP, ADDM addM,
                                                double stb[7], double* s0b) {
    const Cst<double>& K = P.cd;
    const double u = st[0], v = st[1], w = st[2], T = st[3];
    const double nx = st[4] * s0, ny = st[5] * s0, nz = st[6] * s0;
    const bool zy = fabs(nz) <= fabs(ny);
    const double ssq = zy ? nx * nx + ny * ny : nx * nx + nz * nz;
    const double ss = 1.0 / sqrt(ssq);
    const double lx = zy ? -ny * ss : -nz * ss, ly = zy ? nx * ss : 0.0, lz = zy ? 0.0 : nx * ss;
    const double mx = ny * lz - nz * ly, my = nz * lx - nx * lz, mz = nx * ly - ny * lx;
    const double qn = u * nx + v * ny + w * nz, ql = u * lx + v * ly + w * lz, qm = u * mx + v * my + w * mz;
    const double q2 = 0.5 * (u * u + v * v + w * w);
    const double gT = K.grg * T;
    const double rc = 1.0 / sqrt(gT), c = gT * rc, c2 = 0.5 * rc, Kc = K.gm1 * (rc * rc), K2 = 0.5 * Kc;
    const double H = gT * K.inv_gm1 + q2;
    constexpr bool w7 = W7;
    const double tmp = w7 ? 1.0 / 12.0 : 1.0 / 6.0;
    constexpr int np = w7 ? 7 : 5;  // stencil points a side (compile time: the arrays stay in registers)
    auto Lrow = [&](int k, double l[5]) {
        if (k == 0) { l[0] = K2 * q2 + qn * c2; l[1] = -(K2 * u + nx * c2); l[2] = -(K2 * v + ny * c2); l[3] = -(K2 * w + nz * c2); l[4] = K2; }
        else if (k == 1) { l[0] = 1.0 - Kc * q2; l[1] = Kc * u; l[2] = Kc * v; l[3] = Kc * w; l[4] = -Kc; }
        else if (k == 2) { l[0] = K2 * q2 - qn * c2; l[1] = -(K2 * u - nx * c2); l[2] = -(K2 * v - ny * c2); l[3] = -(K2 * w - nz * c2); l[4] = K2; }
        else if (k == 3) { l[0] = -ql; l[1] = lx; l[2] = ly; l[3] = lz; l[4] = 0.0; }
        else { l[0] = -qm; l[1] = mx; l[2] = my; l[3] = mz; l[4] = 0.0; }
    };
    // stencil positions of the two sides, in upwind order
    auto posP = [&](int k) { return w7 ? t + k : t + 1 + k; };
    auto posM = [&](int k) { return w7 ? t + 7 - k : t + 6 - k; };
    // ---- reverse of out = R f (the right eigenvectors, schemes.jl:983-999): the cotangents of
    // the characteristic fluxes f need R only; the terms that need f itself (R's dependence on
    // the face state) are linear in f and added once the field loop has formed each f_k
    const double fb[5] = {
        Fb[0] + Fb[1] * (u - c * nx) + Fb[2] * (v - c * ny) + Fb[3] * (w - c * nz) + Fb[4] * (H - qn * c),
        Fb[0] + Fb[1] * u + Fb[2] * v + Fb[3] * w + Fb[4] * q2,
        Fb[0] + Fb[1] * (u + c * nx) + Fb[2] * (v + c * ny) + Fb[3] * (w + c * nz) + Fb[4] * (H + qn * c),
        Fb[1] * lx + Fb[2] * ly + Fb[3] * lz + Fb[4] * ql,
        Fb[1] * mx + Fb[2] * my + Fb[3] * mz + Fb[4] * qm};
    double f[5];
    double ub = 0.0, vb = 0.0, wb = 0.0, nxb = 0.0, nyb = 0.0, nzb = 0.0, qnb = 0.0, q2b = 0.0;
    double lxb = 0.0, lyb = 0.0, lzb = 0.0, qlb = 0.0, mxb = 0.0, myb = 0.0, mzb = 0.0, qmb = 0.0;
    double K2b = 0.0, Kcb = 0.0, c2b = 0.0, cb = 0.0, Hb = 0.0;
    // ---- reverse of the WENO of each field and of the projections L_k . F
#pragma unroll 1
    for (int k = 0; k < 5; k++) {
        const double g = fb[k] * tmp;
        double l[5];
        Lrow(k, l);
        // the two sides one after the other (fewer live registers): projections L_k . F on the
        // side's stencil, the WENO reverse (with the side's forward value), the cotangents of the
        // split fluxes and of row k of L
        double lb[5] = {0, 0, 0, 0, 0};
        double fs[2];
#pragma unroll
        for (int side = 0; side < 2; side++) {
            double V[np], Vb[np];
#pragma unroll
            for (int j = 0; j < np; j++) {
                const int a = side == 0 ? posP(j) : posM(j);
                V[j] = side == 0 ? FP(0, a) * l[0] + FP(1, a) * l[1] + FP(2, a) * l[2] + FP(3, a) * l[3] + FP(4, a) * l[4]
                                 : FM(0, a) * l[0] + FM(1, a) * l[1] + FM(2, a) * l[2] + FM(3, a) * l[3] + FM(4, a) * l[4];
            }
            if constexpr (W7) weno7_vjp(V, s0, g, Vb, s0b, &fs[side]);
            else weno5_vjp(V, s0, g, Vb, s0b, &fs[side]);
#pragma unroll
            for (int j = 0; j < np; j++) {
                const int a = side == 0 ? posP(j) : posM(j);
#pragma unroll
                for (int e = 0; e < 5; e++) {
                    lb[e] += (side == 0 ? FP(e, a) : FM(e, a)) * Vb[j];
                    if (l[e] != 0.0) {
                        if (side == 0) addP(e, a, l[e] * Vb[j]);
                        else addM(e, a, l[e] * Vb[j]);
                    }
                }
            }
        }
        f[k] = (fs[0] + fs[1]) * tmp;
        // row k of L in terms of the face quantities
        if (k == 0 || k == 2) {
            const double sg = k == 0 ? 1.0 : -1.0;
            K2b += lb[0] * q2 - lb[1] * u - lb[2] * v - lb[3] * w + lb[4];
            q2b += K2 * lb[0];
            qnb += sg * c2 * lb[0];
            c2b += sg * (qn * lb[0] - nx * lb[1] - ny * lb[2] - nz * lb[3]);
            ub -= K2 * lb[1];
            vb -= K2 * lb[2];
            wb -= K2 * lb[3];
            nxb -= sg * c2 * lb[1];
            nyb -= sg * c2 * lb[2];
            nzb -= sg * c2 * lb[3];
        } else if (k == 1) {
            Kcb += -q2 * lb[0] + u * lb[1] + v * lb[2] + w * lb[3] - lb[4];
            q2b -= Kc * lb[0];
            ub += Kc * lb[1];
            vb += Kc * lb[2];
            wb += Kc * lb[3];
        } else if (k == 3) {
            qlb -= lb[0];
            lxb += lb[1];
            lyb += lb[2];
            lzb += lb[3];
        } else {
            qmb -= lb[0];
            mxb += lb[1];
            myb += lb[2];
            mzb += lb[3];
        }
    }
    // R's dependence on the face state (out = R f)
    {
        const double s012 = f[0] + f[1] + f[2], d20 = f[2] - f[0];
        ub += s012 * Fb[1];
        vb += s012 * Fb[2];
        wb += s012 * Fb[3];
        cb += d20 * (nx * Fb[1] + ny * Fb[2] + nz * Fb[3] + qn * Fb[4]);
        nxb += c * d20 * Fb[1];
        nyb += c * d20 * Fb[2];
        nzb += c * d20 * Fb[3];
        qnb += c * d20 * Fb[4];
        Hb += (f[0] + f[2]) * Fb[4];
        q2b += f[1] * Fb[4];
        lxb += f[3] * Fb[1]; lyb += f[3] * Fb[2]; lzb += f[3] * Fb[3]; qlb += f[3] * Fb[4];
        mxb += f[4] * Fb[1]; myb += f[4] * Fb[2]; mzb += f[4] * Fb[3]; qmb += f[4] * Fb[4];
    }
    // ---- the face quantities in terms of (u, v, w, T, n)
    Kcb += 0.5 * K2b;                                  // K2 = Kc / 2
    double rcb = Kcb * K.gm1 * 2.0 * rc + 0.5 * c2b;   // Kc = (g-1) rc^2, c2 = rc / 2
    double gTb = cb * rc + Hb * K.inv_gm1;             // c = gT rc, H = gT/(g-1) + q2
    rcb += cb * gT;
    q2b += Hb;
    gTb += rcb * (-0.5 * rc * rc * rc);                // rc = gT^(-1/2)
    stb[3] += gTb * K.grg;                             // gT = g Rg T
    ub += q2b * u + qnb * nx + qlb * lx + qmb * mx;
    vb += q2b * v + qnb * ny + qlb * ly + qmb * my;
    wb += q2b * w + qnb * nz + qlb * lz + qmb * mz;
    nxb += qnb * u;
    nyb += qnb * v;
    nzb += qnb * w;
    lxb += qlb * u;
    lyb += qlb * v;
    lzb += qlb * w;
    mxb += qmb * u;
    myb += qmb * v;
    mzb += qmb * w;
    // m = n x l
    nyb += mxb * lz; lzb += mxb * ny; nzb -= mxb * ly; lyb -= mxb * nz;
    nzb += myb * lx; lxb += myb * nz; nxb -= myb * lz; lzb -= myb * nx;
    nxb += mzb * ly; lyb += mzb * nx; nyb -= mzb * lx; lxb -= mzb * ny;
    // l from n (the basis branch frozen); ss = ssq^(-1/2)
    const double ss3 = ss * ss * ss;
    if (zy) {  // lx = -ny ss, ly = nx ss
        const double ssb = -ny * lxb + nx * lyb;
        nyb -= lxb * ss;
        nxb += lyb * ss;
        nxb -= ssb * nx * ss3;
        nyb -= ssb * ny * ss3;
    } else {  // lx = -nz ss, lz = nx ss
        const double ssb = -nz * lxb + nx * lzb;
        nzb -= lxb * ss;
        nxb += lzb * ss;
        nxb -= ssb * nx * ss3;
        nzb -= ssb * nz * ss3;
    }
    stb[0] += ub;
    stb[1] += vb;
    stb[2] += wb;
    // n = A s0
    stb[4] += nxb * s0;
    stb[5] += nyb * s0;
    stb[6] += nzb * s0;
    if (s0b) *s0b += nxb * st[4] + nyb * st[5] + nzb * st[6];
}

template <class FPA, class FMA, class ADDP, class ADDM>
__device__ __forceinline__ void char_face_vjp(const DevParams& P, int br, int t, double s0, const double st[7],
                                              const double Fb[5], FPA FP, FMA FM, ADDP addP, ADDM addM,
                                              double stb[7], double* s0b) {
    if (br == 1) char_face_vjp_t<true>(t, P, s0, st, Fb, FP, FM, addP, addM, stb, s0b);
    else char_face_vjp_t<false>(t, P, s0, st, Fb, FP, FM, addP, addM, stb, s0b);
}

}  // namespace f3d
