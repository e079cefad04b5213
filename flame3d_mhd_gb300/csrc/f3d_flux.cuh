// f3d_flux.cuh — per-cell flux splitting and per-face reconstruction, templated on the
// arithmetic type (double for the FP64 drop-in, float for the mixed-precision form).
#pragma once
#include "f3d_common.cuh"

namespace f3d {

// Sign split E+ = max(E,0), E- = min(E,0): equal to (E+|E|)/2 and E-(E+|E|)/2 of
// split.jl:34-40 for every finite E. In FP64 the choice is made on the sign bit with
// integer instructions, keeping it off the FP64 pipe.
__device__ __forceinline__ void sign_split(double e, double& ep, double& em) {
    const bool pos = __double2hiint(e) >= 0;
    ep = pos ? e : 0.0;
    em = pos ? 0.0 : e;
}
__device__ __forceinline__ void sign_split(float e, float& ep, float& em) {
    ep = fmaxf(e, 0.f);
    em = fminf(e, 0.f);
}
__device__ __forceinline__ double rsq(double x) { return rsqrt(x); }
__device__ __forceinline__ float rsq(float x) { return rsqrtf(x); }

// Flux-vector splitting of one cell (split.jl). q = (rho,u,v,w,p,T); A = the J^-1-scaled
// metric row of the sweep direction; Ah = A/|A| (precomputed as A*(1/|A|), split.jl:28-32);
// ss = |A|; c = sound speed (sqrt(gamma Rg T) for SW, split.jl:22; sqrt(gamma p/rho) for
// LF/VL/AUSM, split.jl:90,130,205). Constant quotients such as 1/(2 gamma) and
// (3-gamma)/(2(gamma-1)) come precomputed in K instead of being divided per cell.
template <class R>
__device__ __forceinline__ void split_cell(int method, const Cst<R>& K, const R q[6], R c, R A1, R A2, R A3, R Ah1,
                                           R Ah2, R Ah3, R ss, R fp[5], R fm[5]) {
    const R rho = q[0], u = q[1], v = q[2], w = q[3], p = q[4];
    const R half = R(0.5), one = R(1), two = R(2);
    const R g = K.gamma;
    if (method == F3D_SPLIT_SW && sizeof(R) == 8) {  // split.jl:2-68, FP64 form
        // Equal to the reference's expression up to rounding, in fewer FP64 operations:
        // - the common factor t1 = rho / (2 gamma) > 0 is applied to the three eigenvalues before
        //   their sign split (it keeps each sign, -0 included), so no flux component needs its
        //   own final multiplication;
        // - with the unit normal Ah = A/|A| and the normal velocity Un = Ah.u, E1 = |A| Un, and
        //   the eigenvectors' velocities u -+ c Ah and enthalpies |u -+ c Ah|^2/2 + W2 = H -+ c Un
        //   (|Ah| = 1 and 1/2 + (3-gamma)/(2(gamma-1)) = 1/(gamma-1), so H = |u|^2/2 + c^2/(gamma-1))
        //   are never formed: a velocity component of a side's flux is (its mass flux) u + c
        //   (e3 - e2 of that side) Ah;
        // - the eigenvalues are ordered, e2 = e1 - t1 c|A| < e1 < e3 = e1 + t1 c|A|, so their
        //   signs take one of four patterns: all >= 0 (supersonic towards +), all < 0, or the
        //   subsonic e2 < 0 <= e3 with only e1 free. Each pattern sums just the eigenvalues that
        //   land on a side (the dropped terms are exact zeros); a warp only diverges where its
        //   cells straddle a sonic point.
        // 41 FP64 operations a cell in the subsonic pattern, against 63 for the reference's form.
        const R tss = (rho * ss) * K.inv_2g;  // t1 |A|
        const R Un = Ah1 * u + Ah2 * v + Ah3 * w;
        const R e1 = tss * Un, tcs = tss * c;
        const R e2 = e1 - tcs, e3 = e1 + tcs;
        const R q2 = u * u + v * v + w * w;
        const R vv = K.gm1 * q2;
        const R H = half * q2 + (K.inv_gm1 * c) * c;
        const R cUn = c * Un;
        const bool e2pos = __double2hiint(e2) >= 0, e3pos = __double2hiint(e3) >= 0;
        if (e2pos || !e3pos) {  // every eigenvalue on one side
            const R a1 = K.two_gm1 * e1;
            const R s23 = e2 + e3, d23 = e3 - e2;
            const R f0 = a1 + s23, dc = d23 * c;
            const R f[5] = {f0, f0 * u + dc * Ah1, f0 * v + dc * Ah2, f0 * w + dc * Ah3,
                            e1 * vv + s23 * H + d23 * cUn};
#pragma unroll
            for (int n = 0; n < 5; n++) {
                fp[n] = e2pos ? f[n] : R(0);
                fm[n] = e2pos ? R(0) : f[n];
            }
        } else {  // e2 < 0 <= e3: e2 to Fm, e3 to Fp, e1 by its sign
            R e1p, e1m;
            sign_split(e1, e1p, e1m);
            const R a1 = K.two_gm1 * e1p, b1 = K.two_gm1 * e1m;
            const R fp0 = a1 + e3, e3c = e3 * c;
            const R fm0 = b1 + e2, e2c = e2 * c;
            fp[0] = fp0;
            fp[1] = fp0 * u + e3c * Ah1;
            fp[2] = fp0 * v + e3c * Ah2;
            fp[3] = fp0 * w + e3c * Ah3;
            fp[4] = e1p * vv + e3 * (H + cUn);
            fm[0] = fm0;
            fm[1] = fm0 * u - e2c * Ah1;
            fm[2] = fm0 * v - e2c * Ah2;
            fm[3] = fm0 * w - e2c * Ah3;
            fm[4] = e1m * vv + e2 * (H - cUn);
        }
    } else if (method == F3D_SPLIT_SW) {  // split.jl:2-68
        R E1 = A1 * u + A2 * v + A3 * w;
        R E2 = E1 - c * ss;
        R E3 = E1 + c * ss;
        R E1P, E2P, E3P, E1M, E2M, E3M;
        sign_split(E1, E1P, E1M);
        sign_split(E2, E2P, E2M);
        sign_split(E3, E3P, E3M);
        R uc1 = u - c * Ah1, uc2 = u + c * Ah1;
        R vc1 = v - c * Ah2, vc2 = v + c * Ah2;
        R wc1 = w - c * Ah3, wc2 = w + c * Ah3;
        R vvc1 = (uc1 * uc1 + vc1 * vc1 + wc1 * wc1) * half;
        R vvc2 = (uc2 * uc2 + vc2 * vc2 + wc2 * wc2) * half;
        R vv = K.gm1 * (u * u + v * v + w * w);
        R W2 = K.w2c * (c * c);
        R t1 = rho * K.inv_2g;
        R a1 = K.two_gm1 * E1P, b1 = K.two_gm1 * E1M;
        fp[0] = t1 * (a1 + E2P + E3P);
        fp[1] = t1 * (a1 * u + E2P * uc1 + E3P * uc2);
        fp[2] = t1 * (a1 * v + E2P * vc1 + E3P * vc2);
        fp[3] = t1 * (a1 * w + E2P * wc1 + E3P * wc2);
        fp[4] = t1 * (E1P * vv + E2P * vvc1 + E3P * vvc2 + W2 * (E2P + E3P));
        fm[0] = t1 * (b1 + E2M + E3M);
        fm[1] = t1 * (b1 * u + E2M * uc1 + E3M * uc2);
        fm[2] = t1 * (b1 * v + E2M * vc1 + E3M * vc2);
        fm[3] = t1 * (b1 * w + E2M * wc1 + E3M * wc2);
        fm[4] = t1 * (E1M * vv + E2M * vvc1 + E3M * vvc2 + W2 * (E2M + E3M));
    } else if (method == F3D_SPLIT_LF) {  // split.jl:70-108
        R un = A1 * u + A2 * v + A3 * w;
        R l0 = fabs(un) + c * ss;
        R E0 = p * K.inv_gm1 + half * rho * (u * u + v * v + w * w);
        R ru = rho * u, rv = rho * v, rw = rho * w;
        fp[0] = half * (rho * un + l0 * rho);
        fp[1] = half * (ru * un + A1 * p + l0 * ru);
        fp[2] = half * (rv * un + A2 * p + l0 * rv);
        fp[3] = half * (rw * un + A3 * p + l0 * rw);
        fp[4] = half * ((E0 + p) * un + l0 * E0);
        fm[0] = half * (rho * un - l0 * rho);
        fm[1] = half * (ru * un + A1 * p - l0 * ru);
        fm[2] = half * (rv * un + A2 * p - l0 * rv);
        fm[3] = half * (rw * un + A3 * p - l0 * rw);
        fm[4] = half * ((E0 + p) * un - l0 * E0);
    } else {  // VL split.jl:110-183, AUSM split.jl:185-255
        R un = A1 * u + A2 * v + A3 * w;
        R M = un / (c * ss);
        R kin = u * u + v * v + w * w;
        R f4;  // energy flux of the supersonic state
        R h = R(0);
        if (method == F3D_SPLIT_VL) {
            R E0 = p * K.inv_gm1 + half * rho * kin;
            f4 = (E0 + p) * un;
        } else {
            h = g * p / (rho * K.gm1) + half * kin;
            f4 = rho * h * un;
        }
        if (M <= R(-1) || M >= R(1)) {
            R full[5] = {rho * un, rho * u * un + A1 * p, rho * v * un + A2 * p, rho * w * un + A3 * p, f4};
            const bool neg = M <= R(-1);
            for (int n = 0; n < 5; n++) {
                fp[n] = neg ? R(0) : full[n];
                fm[n] = neg ? full[n] : R(0);
            }
        } else if (method == F3D_SPLIT_VL) {
            R unn = un / ss;
            R f1p = rho * c * R(0.25) * sq(M + one) * ss;
            R f1m = -rho * c * R(0.25) * sq(M - one) * ss;
            R t1 = (-unn + two * c) / (g * ss);
            R t2 = (-unn - two * c) / (g * ss);
            R t3 = one / (two * (g * g - one));
            R t4 = half * (kin - unn * unn);
            fp[0] = f1p;
            fp[1] = f1p * (A1 * t1 + u);
            fp[2] = f1p * (A2 * t1 + v);
            fp[3] = f1p * (A3 * t1 + w);
            fp[4] = f1p * (sq(K.gm1 * unn + two * c) * t3 + t4);
            fm[0] = f1m;
            fm[1] = f1m * (A1 * t2 + u);
            fm[2] = f1m * (A2 * t2 + v);
            fm[3] = f1m * (A3 * t2 + w);
            fm[4] = f1m * (sq(K.gm1 * unn - two * c) * t3 + t4);
        } else {
            R f_p = R(0.25) * sq(M + one) * rho * c * ss;
            R f_m = -R(0.25) * sq(M - one) * rho * c * ss;
            R Pp = p * (R(0.25) * sq(M + one) * (two - M));
            R Pm = p * (R(0.25) * sq(M - one) * (two + M));
            fp[0] = f_p;
            fp[1] = f_p * u + A1 * Pp;
            fp[2] = f_p * v + A2 * Pp;
            fp[3] = f_p * w + A3 * Pp;
            fp[4] = f_p * h;
            fm[0] = f_m;
            fm[1] = f_m * u + A1 * Pm;
            fm[2] = f_m * v + A2 * Pm;
            fm[3] = f_m * w + A3 * Pm;
            fm[4] = f_m * h;
        }
    }
}

// ------------------------------------------------------------------------------------
// Nonlinear weights. The reference normalises alpha_k = d_k / b_k, b_k = (eps + IS_k s)^2
// with one division per alpha plus one for the sum (schemes.jl:178-185, 243-252). The
// combine functions take the bases t_k = eps + IS_k s.
// FP64 form: multiply numerator and denominator by prod_k b_k, leaving ONE division per
// stencil side; with b_k in [eps^2, ~1e40] the products stay far inside the FP64 range.
// FP32 form: scale by the smallest base, r_k = min_j t_j / t_k in (0,1], alpha_k = d_k r_k^2,
// so every scaled alpha lies in [0, d_k] and the sum in [d_min, sum d_k]. This keeps the
// eps = 1e-20 of WENO7 usable in FP32, where 1/(1e-20)^2 overflows (the reason the
// reference promotes these alphas to FP64), and never forms a subnormal.

__device__ __forceinline__ double weno5_combine(double t1, double t2, double t3, double v1, double v2, double v3) {
    double b1 = t1 * t1, b2 = t2 * t2, b3 = t3 * t3;
    double a1 = b2 * b3, a2 = 6.0 * b1 * b3, a3 = 3.0 * b1 * b2;
    return (a1 * v1 + a2 * v2 + a3 * v3) / (a1 + a2 + a3);
}
__device__ __forceinline__ float weno5_combine(float t1, float t2, float t3, float v1, float v2, float v3) {
    float m = fminf(t1, fminf(t2, t3));
    float r1 = m / t1, r2 = m / t2, r3 = m / t3;
    float a1 = r1 * r1, a2 = 6.f * r2 * r2, a3 = 3.f * r3 * r3;
    return (a1 * v1 + a2 * v2 + a3 * v3) / (a1 + a2 + a3);
}
__device__ __forceinline__ double weno7_combine(double t1, double t2, double t3, double t4, double q1, double q2,
                                                double q3, double q4) {
    double b1 = t1 * t1, b2 = t2 * t2, b3 = t3 * t3, b4 = t4 * t4;
    double p12 = b1 * b2, p34 = b3 * b4;
    double a1 = b2 * p34, a2 = 12.0 * b1 * p34, a3 = 18.0 * p12 * b4, a4 = 4.0 * p12 * b3;
    return (a1 * q1 + a2 * q2 + a3 * q3 + a4 * q4) / (a1 + a2 + a3 + a4);
}
__device__ __forceinline__ float weno7_combine(float t1, float t2, float t3, float t4, float q1, float q2, float q3,
                                               float q4) {
    float m = fminf(fminf(t1, t2), fminf(t3, t4));
    float r1 = m / t1, r2 = m / t2, r3 = m / t3, r4 = m / t4;
    float a1 = r1 * r1, a2 = 12.f * r2 * r2, a3 = 18.f * r3 * r3, a4 = 4.f * r4 * r4;
    return (a1 * q1 + a2 * q2 + a3 * q3 + a4 * q4) / (a1 + a2 + a3 + a4);
}

// WENO5 of one side, schemes.jl:233-252: 6x the reconstructed value. V in upwind order.
template <class R> __device__ __forceinline__ R weno5(R V1, R V2, R V3, R V4, R V5, R s0) {
    const R e2 = R(1e-16);
    R s11 = R(13) * sq(V1 - R(2) * V2 + V3) + R(3) * sq(V1 - R(4) * V2 + R(3) * V3);
    R s22 = R(13) * sq(V2 - R(2) * V3 + V4) + R(3) * sq(V2 - V4);
    R s33 = R(13) * sq(V3 - R(2) * V4 + V5) + R(3) * sq(R(3) * V3 - R(4) * V4 + V5);
    R t1 = e2 + s11 * s0, t2 = e2 + s22 * s0, t3 = e2 + s33 * s0;
    R v1 = R(2) * V1 - R(7) * V2 + R(11) * V3;
    R v2 = -V2 + R(5) * V3 + R(2) * V4;
    R v3 = R(2) * V3 + R(5) * V4 - V5;
    return weno5_combine(t1, t2, t3, v1, v2, v3);
}

// WENO7 of one side, schemes.jl:153-185: 12x the reconstructed value.
template <class R>
__device__ __forceinline__ void weno7_parts(R V1, R V2, R V3, R V4, R V5, R V6, R V7, R q[4], R Is[4]) {
    q[0] = R(-3) * V1 + R(13) * V2 - R(23) * V3 + R(25) * V4;
    q[1] = V2 - R(5) * V3 + R(13) * V4 + R(3) * V5;
    q[2] = -V3 + R(7) * V4 + R(7) * V5 - V6;
    q[3] = R(3) * V4 + R(13) * V5 - R(5) * V6 + V7;
    Is[0] = V1 * (R(547) * V1 - R(3882) * V2 + R(4642) * V3 - R(1854) * V4) +
            V2 * (R(7043) * V2 - R(17246) * V3 + R(7042) * V4) + V3 * (R(11003) * V3 - R(9402) * V4) +
            V4 * (R(2107) * V4);
    Is[1] = V2 * (R(267) * V2 - R(1642) * V3 + R(1602) * V4 - R(494) * V5) +
            V3 * (R(2843) * V3 - R(5966) * V4 + R(1922) * V5) + V4 * (R(3443) * V4 - R(2522) * V5) +
            V5 * (R(547) * V5);
    Is[2] = V3 * (R(547) * V3 - R(2522) * V4 + R(1922) * V5 - R(494) * V6) +
            V4 * (R(3443) * V4 - R(5966) * V5 + R(1602) * V6) + V5 * (R(2843) * V5 - R(1642) * V6) +
            V6 * (R(267) * V6);
    Is[3] = V4 * (R(2107) * V4 - R(9402) * V5 + R(7042) * V6 - R(1854) * V7) +
            V5 * (R(11003) * V5 - R(17246) * V6 + R(4642) * V7) + V6 * (R(7043) * V6 - R(3882) * V7) +
            V7 * (R(547) * V7);
}

// The reference's own Float32 forms (F3D_PREC_REF32). WENO7: smoothness indicators and
// stencil values in Float32, the alphas d_k / (1e-20 + IS_k s0)^2 and their normalised
// combination in FP64 (schemes.jl:178-185 promotes them); returns 12x the value in FP64.
__device__ __forceinline__ double weno7_ref32(float V1, float V2, float V3, float V4, float V5, float V6, float V7,
                                              float s0) {
    float q[4], Is[4];
    weno7_parts<float>(V1, V2, V3, V4, V5, V6, V7, q, Is);
    const double e1 = 1e-20;
    const double a1 = 1.0 / sq(e1 + (double)(Is[0] * s0)), a2 = 12.0 / sq(e1 + (double)(Is[1] * s0));
    const double a3 = 18.0 / sq(e1 + (double)(Is[2] * s0)), a4 = 4.0 / sq(e1 + (double)(Is[3] * s0));
    const double invsum = 1.0 / (a1 + a2 + a3 + a4);
    return invsum * (a1 * (double)q[0] + a2 * (double)q[1] + a3 * (double)q[2] + a4 * (double)q[3]);
}
// WENO5 in Float32 with one division per alpha and one for their sum (schemes.jl:233-252).
__device__ __forceinline__ float weno5_ref32(float V1, float V2, float V3, float V4, float V5, float s0) {
    float s11 = 13.f * sq(V1 - 2.f * V2 + V3) + 3.f * sq(V1 - 4.f * V2 + 3.f * V3);
    float s22 = 13.f * sq(V2 - 2.f * V3 + V4) + 3.f * sq(V2 - V4);
    float s33 = 13.f * sq(V3 - 2.f * V4 + V5) + 3.f * sq(3.f * V3 - 4.f * V4 + V5);
    const float e2 = 1e-16f;
    s11 = 1.f / sq(e2 + s11 * s0);
    s22 = 6.f / sq(e2 + s22 * s0);
    s33 = 3.f / sq(e2 + s33 * s0);
    const float invsum = 1.f / (s11 + s22 + s33);
    const float v1 = 2.f * V1 - 7.f * V2 + 11.f * V3, v2 = -V2 + 5.f * V3 + 2.f * V4, v3 = 2.f * V3 + 5.f * V4 - V5;
    return invsum * (s11 * v1 + s22 * v2 + s33 * v3);
}

// WENO7 smoothness indicators in difference form. The reference writes IS_k as a quadratic
// form in the stencil values (schemes.jl:160-175, e.g. IS_1 = V1 (547 V1 - 3882 V2 + ...) + ...);
// IS_k vanishes on constants, so it is a quadratic form in the first differences
// d_j = V_{k+j} - V_{k+j-1} of its sub-stencil, and the LDL^T factorisation of that 3 x 3 form
// writes it as a positively weighted sum of squares:
//   IS_k = D1 (d1 + a d2 + b d3)^2 + D2 (d2 + c d3)^2 + D3 d3^2,
// equal to the reference's expression in exact arithmetic. Evaluated in floating point the
// expanded form cancels terms of size 1e4 V^2 down to IS ~ (V differences)^2: on a stencil of
// values ~1 varying by 1e-3 its relative rounding error reaches 1e-9 in FP64 and 0.5 in FP32,
// while the difference form stays within a few ulps (and is never negative). Fewer operations,
// too. Constants per sub-stencil k: {D1, a, b, D2, c, D3}.
template <class R> struct W7Ldl;
#define F3D_W7LDL(T)                                                                                          \
    template <> struct W7Ldl<T> {                                                                            \
        static __device__ __forceinline__ T D1(int k) { return k == 0 ? T(547) : k == 1 ? T(267) : k == 2 ? T(547) : T(2107); } \
        static __device__ __forceinline__ T a(int k) {                                                        \
            return k == 0 ? T(-1394.0 / 547.0) : k == 1 ? T(-554.0 / 267.0) : k == 2 ? T(-714.0 / 547.0) : T(-2594.0 / 2107.0); \
        }                                                                                                     \
        static __device__ __forceinline__ T b(int k) {                                                        \
            return k == 0 ? T(927.0 / 547.0) : k == 1 ? T(247.0 / 267.0) : k == 2 ? T(247.0 / 547.0) : T(927.0 / 2107.0); \
        }                                                                                                     \
        static __device__ __forceinline__ T D2(int k) {                                                       \
            return k == 0 ? T(85040.0 / 547.0) : k == 1 ? T(85040.0 / 267.0) : k == 2 ? T(293200.0 / 547.0) : T(1083920.0 / 2107.0); \
        }                                                                                                     \
        static __device__ __forceinline__ T c(int k) {                                                        \
            return k == 0 ? T(-3167.0 / 2126.0) : k == 1 ? T(-1345.0 / 2126.0) : k == 2 ? T(-3167.0 / 7330.0) : T(-13313.0 / 27098.0); \
        }                                                                                                     \
        static __device__ __forceinline__ T D3(int k) {                                                       \
            return k == 0 ? T(203060.0 / 1063.0) : k == 1 ? T(203060.0 / 1063.0) : k == 2 ? T(40612.0 / 733.0) : T(203060.0 / 13549.0); \
        }                                                                                                     \
    };
F3D_W7LDL(double)
F3D_W7LDL(float)
#undef F3D_W7LDL

template <class R> __device__ __forceinline__ void weno7_is(const R V[7], R Is[4]) {
    using C = W7Ldl<R>;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const R d1 = V[k + 1] - V[k], d2 = V[k + 2] - V[k + 1], d3 = V[k + 3] - V[k + 2];
        const R y1 = d1 + C::a(k) * d2 + C::b(k) * d3, y2 = d2 + C::c(k) * d3;
        Is[k] = C::D1(k) * (y1 * y1) + C::D2(k) * (y2 * y2) + C::D3(k) * (d3 * d3);
    }
}

// WENO7 of one side, schemes.jl:153-185: 12x the reconstructed value (FP64 and mixed forms;
// the smoothness indicators in the difference form above).
template <class R> __device__ __forceinline__ R weno7(R V1, R V2, R V3, R V4, R V5, R V6, R V7, R s0) {
    R q1 = R(-3) * V1 + R(13) * V2 - R(23) * V3 + R(25) * V4;
    R q2 = V2 - R(5) * V3 + R(13) * V4 + R(3) * V5;
    R q3 = -V3 + R(7) * V4 + R(7) * V5 - V6;
    R q4 = R(3) * V4 + R(13) * V5 - R(5) * V6 + V7;
    const R V[7] = {V1, V2, V3, V4, V5, V6, V7};
    R Is[4];
    weno7_is<R>(V, Is);
    const R e1 = R(1e-20);
    return weno7_combine(e1 + Is[0] * s0, e1 + Is[1] * s0, e1 + Is[2] * s0, e1 + Is[3] * s0, q1, q2, q3, q4);
}

}  // namespace f3d
