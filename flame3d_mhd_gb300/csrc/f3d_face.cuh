// f3d_face.cuh — the per-face reconstruction of the finite-difference sweeps (UP7, NND2,
// component- and characteristic-wise WENO7 / WENO5; schemes.jl:86-1643) and the split's sound
// speed, shared by the direct-load sweeps (k_sweep.cu) and the TMA-staged ones
// (k_sweep_tma.cu).
#pragma once
#include "f3d_kernels.cuh"

namespace f3d {

// ---- Characteristic-wise reconstruction, schemes.jl:756-999, in three parts: the face's basis,
// one field's characteristic flux, one component of the face flux. The face's eigenvectors
// come from the arithmetic mean of u, v, w, T and of the metric row at the two adjacent cells
// (cl, cr linear indices), read from global memory. Rows of L and of R are selected by a
// runtime index, and the field loop is not unrolled: one copy of the WENO code serves the
// five fields (the FP64 characteristic sweeps hold 96 registers with no spills this way).
// Spreading a face over five lanes, one field each, with the fluxes exchanged by shuffles
// ran 7.5% slower per RK3 step on the 256x64x64 shock tube than one thread per face: the
// five copies of the basis cost more than the idle lanes of a short WENO queue.
template <class R> struct CharBasis {
    R u, v, w, c, q2, H, qn, ql, qm, nx, ny, nz, lx, ly, lz, mx, my, mz, c2, K2, Kc;
};

template <class R>
__device__ __forceinline__ void char_basis(const DevParams& P, const SweepArgs& a, R s0, long long cl, long long cr,
                                           CharBasis<R>& b) {
    const Cst<R>& K = cst<R>(P);
    const long long pl = P.plane;
    const R* Qr = static_cast<const R*>(a.Q);
    const R* A0 = static_cast<const R*>(a.A[0]);
    const R* A1p = static_cast<const R*>(a.A[1]);
    const R* A2p = static_cast<const R*>(a.A[2]);
    const R u = R(0.5) * (Qr[cr + pl] + Qr[cl + pl]);
    const R v = R(0.5) * (Qr[cr + 2 * pl] + Qr[cl + 2 * pl]);
    const R w = R(0.5) * (Qr[cr + 3 * pl] + Qr[cl + 3 * pl]);
    const R T = R(0.5) * (Qr[cr + 5 * pl] + Qr[cl + 5 * pl]);
    const R A1 = (A0[cr] + A0[cl]) * R(0.5);
    const R A2 = (A1p[cr] + A1p[cl]) * R(0.5);
    const R A3 = (A2p[cr] + A2p[cl]) * R(0.5);
    const R nx = A1 * s0, ny = A2 * s0, nz = A3 * s0;
    R lx, ly, lz;
    if (fabs(nz) <= fabs(ny)) {
        R ss = rsq(nx * nx + ny * ny);
        lx = -ny * ss;
        ly = nx * ss;
        lz = R(0);
    } else {
        R ss = rsq(nx * nx + nz * nz);
        lx = -nz * ss;
        ly = R(0);
        lz = nx * ss;
    }
    const R mx = ny * lz - nz * ly, my = nz * lx - nx * lz, mz = nx * ly - ny * lx;
    b.u = u; b.v = v; b.w = w;
    b.nx = nx; b.ny = ny; b.nz = nz;
    b.lx = lx; b.ly = ly; b.lz = lz;
    b.mx = mx; b.my = my; b.mz = mz;
    b.qn = u * nx + v * ny + w * nz;
    b.ql = u * lx + v * ly + w * lz;
    b.qm = u * mx + v * my + w * mz;
    b.q2 = R(0.5) * (u * u + v * v + w * w);
    const R gT = K.grg * T;
    const R rc = rsq(gT);                // 1/c
    b.c = gT * rc;                       // c = sqrt(gamma Rg T)
    b.c2 = R(0.5) * rc;                  // 1/(2c)
    b.Kc = K.gm1 * (rc * rc);            // (gamma-1)/c^2
    b.K2 = b.Kc * R(0.5);
    b.H = gT * K.inv_gm1 + b.q2;         // 1/K + q2
}

// Row n of the left eigenvectors L (schemes.jl:800-830), written for a runtime n as
// alpha_n (q2, -u, -v, -w, 1) + beta_n t_n + (n == 1) e_0 with t_n = (qn, -n) for the
// acoustic rows 0 and 2 (beta = +-1/(2c), alpha = K2), (-ql, l) and (-qm, m) for the shear
// rows 3 and 4 (beta = 1, alpha = 0), and alpha = -Kc, beta = 0 for the entropy row 1.
template <class R>
__device__ __forceinline__ void char_left_row(const CharBasis<R>& b, int n, R l[5]) {
    const R al = n == 0 || n == 2 ? b.K2 : n == 1 ? -b.Kc : R(0);
    const R be = n == 0 ? b.c2 : n == 2 ? -b.c2 : n == 1 ? R(0) : R(1);
    const R t0 = n <= 2 ? b.qn : n == 3 ? -b.ql : -b.qm;
    const R t1 = n <= 2 ? -b.nx : n == 3 ? b.lx : b.mx;
    const R t2 = n <= 2 ? -b.ny : n == 3 ? b.ly : b.my;
    const R t3 = n <= 2 ? -b.nz : n == 3 ? b.lz : b.mz;
    l[0] = al * b.q2 + be * t0 + (n == 1 ? R(1) : R(0));
    l[1] = be * t1 - al * b.u;
    l[2] = be * t2 - al * b.v;
    l[3] = be * t3 - al * b.w;
    l[4] = al;
}

// The characteristic flux of field n at the face: the field's projection L_n F of the stencil's
// split fluxes, reconstructed by WENO7 (br 1) or WENO5 (br 2) on each side.
template <class R, class FPA, class FMA>
__device__ __forceinline__ R char_field_flux(const DevParams& P, const CharBasis<R>& b, int n, int br, int p0, R s0,
                                             FPA FP, FMA FM) {
    const R tmp1 = R(1) / R(12), tmp2 = R(1) / R(6);
    R l[5];
    char_left_row<R>(b, n, l);
    auto projP = [&](int pos) {
        return FP(0, pos) * l[0] + FP(1, pos) * l[1] + FP(2, pos) * l[2] + FP(3, pos) * l[3] + FP(4, pos) * l[4];
    };
    auto projM = [&](int pos) {
        return FM(0, pos) * l[0] + FM(1, pos) * l[1] + FM(2, pos) * l[2] + FM(3, pos) * l[3] + FM(4, pos) * l[4];
    };
    if constexpr (sizeof(R) == 4) {
        if (P.ref32) {  // the reference's Float32 reconstruction of the characteristic fields
            if (br == 1) {
                const double fp = weno7_ref32(projP(p0), projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4),
                                              projP(p0 + 5), projP(p0 + 6), s0);
                const double fm = weno7_ref32(projM(p0 + 7), projM(p0 + 6), projM(p0 + 5), projM(p0 + 4),
                                              projM(p0 + 3), projM(p0 + 2), projM(p0 + 1), s0);
                return (float)((fp + fm) * (double)tmp1);
            }
            return (weno5_ref32(projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4), projP(p0 + 5), s0) +
                    weno5_ref32(projM(p0 + 6), projM(p0 + 5), projM(p0 + 4), projM(p0 + 3), projM(p0 + 2), s0)) *
                   tmp2;
        }
    }
    if (br == 1) {
        R fp = weno7(projP(p0), projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4), projP(p0 + 5),
                     projP(p0 + 6), s0);
        R fm = weno7(projM(p0 + 7), projM(p0 + 6), projM(p0 + 5), projM(p0 + 4), projM(p0 + 3), projM(p0 + 2),
                     projM(p0 + 1), s0);
        return (fp + fm) * tmp1;
    }
    R fp = weno5(projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4), projP(p0 + 5), s0);
    R fm = weno5(projM(p0 + 6), projM(p0 + 5), projM(p0 + 4), projM(p0 + 3), projM(p0 + 2), s0);
    return (fp + fm) * tmp2;
}

// Component k of the face flux R f from the five characteristic fluxes (schemes.jl:960-999):
// f0 (a - c n) + f1 a' + f2 (a + c n) + f3 l + f4 m with (a, a', n, l, m) the k-th entries of
// (1, u, v, w, H), (1, u, v, w, q2), (0, nx, ny, nz, qn), (0, lx, ly, lz, ql), (0, mx, my, mz, qm).
template <class R>
__device__ __forceinline__ R char_right_row(const CharBasis<R>& b, int k, const R f[5]) {
    if (k == 0) return f[0] + f[1] + f[2];
    const R ak = k == 1 ? b.u : k == 2 ? b.v : k == 3 ? b.w : b.H;
    const R ap = k == 4 ? b.q2 : ak;
    const R nk = k == 1 ? b.nx : k == 2 ? b.ny : k == 3 ? b.nz : b.qn;
    const R lk = k == 1 ? b.lx : k == 2 ? b.ly : k == 3 ? b.lz : b.ql;
    const R mk = k == 1 ? b.mx : k == 2 ? b.my : k == 3 ? b.mz : b.qm;
    return f[0] * (ak - b.c * nk) + f[1] * ap + f[2] * (ak + b.c * nk) + f[3] * lk + f[4] * mk;
}

// Face flux of one face from the split fluxes of the 8 cells around it, positions
// p0..p0+7 of the line (face between positions p0+3 and p0+4). FP/FM(n, pos) read shared
// memory. For characteristic mode the face state comes from global memory at the two
// adjacent cells (cl, cr linear indices).
template <bool CHAR, class R, class FPA, class FMA>
__device__ __forceinline__ void face_flux(const DevParams& P, const SweepArgs& a, int br, int p0, R s0,
                                          long long cl, long long cr, FPA FP, FMA FM, R out[5]) {
    const Cst<R>& K = cst<R>(P);
    if (br == 0) {  // UP7, schemes.jl:119-142
        const R c1 = K.lin[0], c2 = K.lin[1], c3 = K.lin[2], c4 = K.lin[3], c5 = K.lin[4], c6 = K.lin[5],
                c7 = K.lin[6];
#pragma unroll
        for (int n = 0; n < 5; n++) {
            if constexpr (sizeof(R) == 8) {
                // FP64: each Fp with its mirrored Fm under one coefficient (14 operations, not 15)
                out[n] = c1 * (FP(n, p0) + FM(n, p0 + 7)) + c2 * (FP(n, p0 + 1) + FM(n, p0 + 6)) +
                         c3 * (FP(n, p0 + 2) + FM(n, p0 + 5)) + c4 * (FP(n, p0 + 3) + FM(n, p0 + 4)) +
                         c5 * (FP(n, p0 + 4) + FM(n, p0 + 3)) + c6 * (FP(n, p0 + 5) + FM(n, p0 + 2)) +
                         c7 * (FP(n, p0 + 6) + FM(n, p0 + 1));
            } else {
                R fp = c1 * FP(n, p0) + c2 * FP(n, p0 + 1) + c3 * FP(n, p0 + 2) + c4 * FP(n, p0 + 3) +
                       c5 * FP(n, p0 + 4) + c6 * FP(n, p0 + 5) + c7 * FP(n, p0 + 6);
                R fm = c1 * FM(n, p0 + 7) + c2 * FM(n, p0 + 6) + c3 * FM(n, p0 + 5) + c4 * FM(n, p0 + 4) +
                       c5 * FM(n, p0 + 3) + c6 * FM(n, p0 + 2) + c7 * FM(n, p0 + 1);
                out[n] = fp + fm;
            }
        }
        return;
    }
    if (br == 3) {  // NND2, schemes.jl:277-286 (component-wise in both modes)
#pragma unroll
        for (int n = 0; n < 5; n++) {
            R fp = FP(n, p0 + 3) + R(0.5) * minmod(FP(n, p0 + 4) - FP(n, p0 + 3), FP(n, p0 + 3) - FP(n, p0 + 2));
            R fm = FM(n, p0 + 4) - R(0.5) * minmod(FM(n, p0 + 5) - FM(n, p0 + 4), FM(n, p0 + 4) - FM(n, p0 + 3));
            out[n] = fp + fm;
        }
        return;
    }
    const R tmp1 = R(1) / R(12), tmp2 = R(1) / R(6);
    if (!CHAR) {  // component-wise WENO7 (schemes.jl:143-230) / WENO5 (:231-276)
#pragma unroll 1
        for (int n = 0; n < 5; n++) {
            if constexpr (sizeof(R) == 4) {
                if (P.ref32) {  // the reference's Float32 reconstruction
                    if (br == 1) {
                        const double fp = weno7_ref32(FP(n, p0), FP(n, p0 + 1), FP(n, p0 + 2), FP(n, p0 + 3),
                                                      FP(n, p0 + 4), FP(n, p0 + 5), FP(n, p0 + 6), s0);
                        const double fm = weno7_ref32(FM(n, p0 + 7), FM(n, p0 + 6), FM(n, p0 + 5), FM(n, p0 + 4),
                                                      FM(n, p0 + 3), FM(n, p0 + 2), FM(n, p0 + 1), s0);
                        out[n] = (float)((fp + fm) * (double)tmp1);
                    } else {
                        out[n] = (weno5_ref32(FP(n, p0 + 1), FP(n, p0 + 2), FP(n, p0 + 3), FP(n, p0 + 4),
                                              FP(n, p0 + 5), s0) +
                                  weno5_ref32(FM(n, p0 + 6), FM(n, p0 + 5), FM(n, p0 + 4), FM(n, p0 + 3),
                                              FM(n, p0 + 2), s0)) *
                                 tmp2;
                    }
                    continue;
                }
            }
            if (br == 1) {
                R fp = weno7(FP(n, p0), FP(n, p0 + 1), FP(n, p0 + 2), FP(n, p0 + 3), FP(n, p0 + 4), FP(n, p0 + 5),
                             FP(n, p0 + 6), s0);
                R fm = weno7(FM(n, p0 + 7), FM(n, p0 + 6), FM(n, p0 + 5), FM(n, p0 + 4), FM(n, p0 + 3),
                             FM(n, p0 + 2), FM(n, p0 + 1), s0);
                out[n] = (fp + fm) * tmp1;
            } else {
                R fp = weno5(FP(n, p0 + 1), FP(n, p0 + 2), FP(n, p0 + 3), FP(n, p0 + 4), FP(n, p0 + 5), s0);
                R fm = weno5(FM(n, p0 + 6), FM(n, p0 + 5), FM(n, p0 + 4), FM(n, p0 + 3), FM(n, p0 + 2), s0);
                out[n] = (fp + fm) * tmp2;
            }
        }
        return;
    }
    // characteristic-wise, schemes.jl:756-999
    CharBasis<R> cb;
    char_basis<R>(P, a, s0, cl, cr, cb);
    R flux[5];
#pragma unroll 1
    for (int n = 0; n < 5; n++) flux[n] = char_field_flux<R>(P, cb, n, br, p0, s0, FP, FM);
#pragma unroll
    for (int k = 0; k < 5; k++) out[k] = char_right_row<R>(cb, k, flux);
}

// Sound speed for the split: precomputed per cell in FP64; computed in place in FP32.
template <class R> __device__ __forceinline__ R split_sound(const DevParams& P, const SweepArgs& a, long long c,
                                                            const R q[6]);
template <> __device__ __forceinline__ double split_sound<double>(const DevParams&, const SweepArgs& a, long long c,
                                                                  const double*) {
    return static_cast<const double*>(a.csnd)[c];
}
template <> __device__ __forceinline__ float split_sound<float>(const DevParams& P, const SweepArgs&, long long,
                                                                const float* q) {
    return P.split == F3D_SPLIT_SW ? sqrtf(P.cf.grg * q[5]) : sqrtf(P.cf.gamma * q[4] / q[0]);
}

}  // namespace f3d
