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
__device__ __forceinline__ void split_sw_vjp(const Cst<double>& K, const double q[6], double c, double A1, double A2,
                                             double A3, double H1, double H2, double H3, double ss,
                                             const double fpb[5], const double fmb[5], double qb[6],
                                             double* mg = nullptr) {
    const double rho = q[0], u = q[1], v = q[2], w = q[3];
    const double E1 = A1 * u + A2 * v + A3 * w;
    const double E[3] = {E1, E1 - c * ss, E1 + c * ss};
    double EP[3], EM[3];
    for (int k = 0; k < 3; k++) sign_split(E[k], EP[k], EM[k]);
    const double uc[2] = {u - c * H1, u + c * H1}, vc[2] = {v - c * H2, v + c * H2}, wc[2] = {w - c * H3, w + c * H3};
    const double vvc[2] = {0.5 * (uc[0] * uc[0] + vc[0] * vc[0] + wc[0] * wc[0]),
                           0.5 * (uc[1] * uc[1] + vc[1] * vc[1] + wc[1] * wc[1])};
    const double vv = K.gm1 * (u * u + v * v + w * w);
    const double W2 = K.w2c * c * c;
    const double t1 = rho * K.inv_2g, t2 = K.two_gm1;
    double t1b = 0, ub = 0, vb = 0, wb = 0, cb = 0, vvb = 0, W2b = 0;
    double Eb[3] = {0, 0, 0};
    double ucb[2] = {0, 0}, vcb[2] = {0, 0}, wcb[2] = {0, 0}, vvcb[2] = {0, 0};
    for (int side = 0; side < 2; side++) {
        const double* g = side == 0 ? fpb : fmb;
        const double* e = side == 0 ? EP : EM;
        // brackets B_n with f_n = t1 * B_n
        const double B0 = t2 * e[0] + e[1] + e[2];
        const double B1 = t2 * e[0] * u + e[1] * uc[0] + e[2] * uc[1];
        const double B2 = t2 * e[0] * v + e[1] * vc[0] + e[2] * vc[1];
        const double B3 = t2 * e[0] * w + e[1] * wc[0] + e[2] * wc[1];
        const double B4 = e[0] * vv + e[1] * vvc[0] + e[2] * vvc[1] + W2 * (e[1] + e[2]);
        t1b += g[0] * B0 + g[1] * B1 + g[2] * B2 + g[3] * B3 + g[4] * B4;
        const double b0 = t1 * g[0], b1 = t1 * g[1], b2 = t1 * g[2], b3 = t1 * g[3], b4 = t1 * g[4];
        double eb0 = t2 * (b0 + u * b1 + v * b2 + w * b3) + vv * b4;
        double eb1 = b0 + uc[0] * b1 + vc[0] * b2 + wc[0] * b3 + (vvc[0] + W2) * b4;
        double eb2 = b0 + uc[1] * b1 + vc[1] * b2 + wc[1] * b3 + (vvc[1] + W2) * b4;
        ub += t2 * e[0] * b1;
        vb += t2 * e[0] * b2;
        wb += t2 * e[0] * b3;
        ucb[0] += e[1] * b1; ucb[1] += e[2] * b1;
        vcb[0] += e[1] * b2; vcb[1] += e[2] * b2;
        wcb[0] += e[1] * b3; wcb[1] += e[2] * b3;
        vvb += e[0] * b4;
        vvcb[0] += e[1] * b4;
        vvcb[1] += e[2] * b4;
        W2b += (e[1] + e[2]) * b4;
        // E+ = max(E,0), E- = min(E,0): each passes its cotangent to E on its own side
        const double ebs[3] = {eb0, eb1, eb2};
        for (int k = 0; k < 3; k++) {
            const bool pos = __double2hiint(E[k]) >= 0;
            Eb[k] += (side == 0) == pos ? ebs[k] : 0.0;
        }
    }
    double rhob = t1b * K.inv_2g;
    cb += W2b * K.w2c * 2.0 * c;
    ub += vvb * K.gm1 * 2.0 * u;
    vb += vvb * K.gm1 * 2.0 * v;
    wb += vvb * K.gm1 * 2.0 * w;
    for (int s = 0; s < 2; s++) {
        ucb[s] += vvcb[s] * uc[s];
        vcb[s] += vvcb[s] * vc[s];
        wcb[s] += vvcb[s] * wc[s];
    }
    ub += ucb[0] + ucb[1];
    vb += vcb[0] + vcb[1];
    wb += wcb[0] + wcb[1];
    cb += (ucb[1] - ucb[0]) * H1 + (vcb[1] - vcb[0]) * H2 + (wcb[1] - wcb[0]) * H3;
    // E2 = E1 - c ss, E3 = E1 + c ss
    const double E1b = Eb[0] + Eb[1] + Eb[2];
    cb += (Eb[2] - Eb[1]) * ss;
    if (mg) {  // E1 = A . u; uc = u -+ c H; E2, E3 = E1 -+ c ss
        mg[0] += E1b * u;
        mg[1] += E1b * v;
        mg[2] += E1b * w;
        mg[3] += (ucb[1] - ucb[0]) * c;
        mg[4] += (vcb[1] - vcb[0]) * c;
        mg[5] += (wcb[1] - wcb[0]) * c;
        mg[6] += (Eb[2] - Eb[1]) * c;
    }
    ub += A1 * E1b;
    vb += A2 * E1b;
    wb += A3 * E1b;
    qb[0] += rhob;
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

// ---- WENO reconstructions: cotangents of the stencil values ---------------------------
// The reference normalises alpha_k = d_k / t_k^2, t_k = eps + IS_k s0, f = sum alpha q / sum alpha
// (schemes.jl:153-185, 233-252). With fb the cotangent of f (already divided by 12 or 6):
// qb_k = fb w_k, alphab_k = fb (q_k - f) / sum alpha, tb_k = -2 alpha_k / t_k alphab_k, and
// IS_k is a quadratic form whose gradient is formed from the coefficient table.
// s0b (optional): += the cotangent of the scale s0 (t_k = eps + IS_k s0).
__device__ __forceinline__ void weno5_vjp(const double V[5], double s0, double fb, double Vb[5],
                                          double* s0b = nullptr) {
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
                                          double* s0b = nullptr) {
    const double d[4] = {1.0, 12.0, 18.0, 4.0};
    double q[4], t[4], IS[4];
    for (int k = 0; k < 4; k++) {
        double is = 0, qq = 0;
        for (int i = 0; i < 4; i++) {
            qq += kW7Q[k][i] * V[k + i];
            for (int j = i; j < 4; j++) is += kW7IS[k][i][j] * V[k + i] * V[k + j];
        }
        q[k] = qq;
        IS[k] = is;
        t[k] = 1e-20 + is * s0;
    }
    // two FP64 divisions: 1/t_k from 1/(t1 t2 t3 t4), and 1/sum alpha
    const double t01 = t[0] * t[1], t23 = t[2] * t[3], rall = 1.0 / (t01 * t23);
    const double it[4] = {t[1] * t23 * rall, t[0] * t23 * rall, t01 * t[3] * rall, t01 * t[2] * rall};
    double al[4], sum = 0;
    for (int k = 0; k < 4; k++) {
        al[k] = d[k] * it[k] * it[k];
        sum += al[k];
    }
    const double rs = 1.0 / sum;
    double f = 0;
    for (int k = 0; k < 4; k++) f += al[k] * rs * q[k];
    for (int j = 0; j < 7; j++) Vb[j] = 0.0;
    for (int k = 0; k < 4; k++) {
        const double wk = al[k] * rs;
        const double qb = fb * wk;
        const double tb = -2.0 * fb * (q[k] - f) * wk * it[k];
        const double ISb = s0 * tb;
        if (s0b) *s0b += IS[k] * tb;
        for (int i = 0; i < 4; i++) {
            Vb[k + i] += kW7Q[k][i] * qb;
            double g = 0;  // dIS/dV_{k+i}
            for (int j = 0; j < 4; j++) {
                if (j >= i) g += kW7IS[k][i][j] * V[k + j];
                if (j <= i) g += kW7IS[k][j][i] * V[k + j];
            }
            Vb[k + i] += g * ISb;
        }
    }
}

}  // namespace f3d
