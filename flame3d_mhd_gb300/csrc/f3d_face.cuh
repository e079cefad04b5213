// f3d_face.cuh — the per-face reconstruction of the finite-difference sweeps (UP7, NND2,
// component- and characteristic-wise WENO7 / WENO5; schemes.jl:86-1643) and the split's sound
// speed, shared by the direct-load sweeps (k_sweep.cu) and the TMA-staged ones
// (k_sweep_tma.cu).
#pragma once
#include "f3d_kernels.cuh"

namespace f3d {

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
    // characteristic-wise, schemes.jl:756-999: eigenvectors of the face from the arithmetic
    // mean of u,v,w,T and of the metric row at the two adjacent cells.
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
    const R qn = u * nx + v * ny + w * nz;
    const R ql = u * lx + v * ly + w * lz;
    const R qm = u * mx + v * my + w * mz;
    const R q2 = R(0.5) * (u * u + v * v + w * w);
    const R gT = K.grg * T;
    const R rc = rsq(gT);              // 1/c
    const R c = gT * rc;               // c = sqrt(gamma Rg T)
    const R c2 = R(0.5) * rc;          // 1/(2c)
    const R Kc = K.gm1 * (rc * rc);    // (gamma-1)/c^2
    const R K2 = Kc * R(0.5);
    const R H = gT * K.inv_gm1 + q2;   // 1/K + q2
    R flux[5];
#pragma unroll 1
    for (int n = 0; n < 5; n++) {
        R l0, l1, l2, l3, l4;  // row n of L
        if (n == 0) { l0 = K2 * q2 + qn * c2; l1 = -(K2 * u + nx * c2); l2 = -(K2 * v + ny * c2); l3 = -(K2 * w + nz * c2); l4 = K2; }
        else if (n == 1) { l0 = R(1) - Kc * q2; l1 = Kc * u; l2 = Kc * v; l3 = Kc * w; l4 = -Kc; }
        else if (n == 2) { l0 = K2 * q2 - qn * c2; l1 = -(K2 * u - nx * c2); l2 = -(K2 * v - ny * c2); l3 = -(K2 * w - nz * c2); l4 = K2; }
        else if (n == 3) { l0 = -ql; l1 = lx; l2 = ly; l3 = lz; l4 = R(0); }
        else { l0 = -qm; l1 = mx; l2 = my; l3 = mz; l4 = R(0); }
        auto projP = [&](int pos) {
            return FP(0, pos) * l0 + FP(1, pos) * l1 + FP(2, pos) * l2 + FP(3, pos) * l3 + FP(4, pos) * l4;
        };
        auto projM = [&](int pos) {
            return FM(0, pos) * l0 + FM(1, pos) * l1 + FM(2, pos) * l2 + FM(3, pos) * l3 + FM(4, pos) * l4;
        };
        if constexpr (sizeof(R) == 4) {
            if (P.ref32) {  // the reference's Float32 reconstruction of the characteristic fields
                if (br == 1) {
                    const double fp = weno7_ref32(projP(p0), projP(p0 + 1), projP(p0 + 2), projP(p0 + 3),
                                                  projP(p0 + 4), projP(p0 + 5), projP(p0 + 6), s0);
                    const double fm = weno7_ref32(projM(p0 + 7), projM(p0 + 6), projM(p0 + 5), projM(p0 + 4),
                                                  projM(p0 + 3), projM(p0 + 2), projM(p0 + 1), s0);
                    flux[n] = (float)((fp + fm) * (double)tmp1);
                } else {
                    flux[n] = (weno5_ref32(projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4),
                                           projP(p0 + 5), s0) +
                               weno5_ref32(projM(p0 + 6), projM(p0 + 5), projM(p0 + 4), projM(p0 + 3),
                                           projM(p0 + 2), s0)) *
                              tmp2;
                }
                continue;
            }
        }
        if (br == 1) {
            R fp = weno7(projP(p0), projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4), projP(p0 + 5),
                         projP(p0 + 6), s0);
            R fm = weno7(projM(p0 + 7), projM(p0 + 6), projM(p0 + 5), projM(p0 + 4), projM(p0 + 3), projM(p0 + 2),
                         projM(p0 + 1), s0);
            flux[n] = (fp + fm) * tmp1;
        } else {
            R fp = weno5(projP(p0 + 1), projP(p0 + 2), projP(p0 + 3), projP(p0 + 4), projP(p0 + 5), s0);
            R fm = weno5(projM(p0 + 6), projM(p0 + 5), projM(p0 + 4), projM(p0 + 3), projM(p0 + 2), s0);
            flux[n] = (fp + fm) * tmp2;
        }
    }
    out[0] = flux[0] + flux[1] + flux[2];
    out[1] = flux[0] * (u - c * nx) + flux[1] * u + flux[2] * (u + c * nx) + flux[3] * lx + flux[4] * mx;
    out[2] = flux[0] * (v - c * ny) + flux[1] * v + flux[2] * (v + c * ny) + flux[3] * ly + flux[4] * my;
    out[3] = flux[0] * (w - c * nz) + flux[1] * w + flux[2] * (w + c * nz) + flux[3] * lz + flux[4] * mz;
    out[4] = flux[0] * (H - qn * c) + flux[1] * q2 + flux[2] * (H + qn * c) + flux[3] * ql + flux[4] * qm;
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
