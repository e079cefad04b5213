// f3d_sweep_epilogue.cuh — pieces shared by the finite-difference and finite-volume
// sweeps: the face branch from the sensor (branch_of) and Phase C: per interior cell of the tile, the difference of its two face fluxes (held in
// shared memory), the CD4 derivative of the viscous flux along the sweep (div.jl:14-48)
// and the accumulation selected by out_mode (OUT_SET / OUT_ADD into acc, OUT_RHS = J *
// (acc + d), OUT_STAGE = the RK update of div.jl plus linComb, utils.jl:57-70).
#pragma once
#include "f3d_kernels.cuh"

namespace f3d {

// Branch of a face from the sensor values of cells i-3..i+2 (schemes.jl:112-117 and
// :119, :143, :231): the FP64 values compare as bit patterns (see DevParams::phib), FP32
// values directly. NaN fails every comparison and selects NND2, like the reference.
__device__ __forceinline__ int branch_of(const DevParams& P, const double* ph) {
    unsigned long long m = __double_as_longlong(ph[0]);
#pragma unroll
    for (int o = 1; o < 6; o++) {
        unsigned long long b = __double_as_longlong(ph[o]);
        m = b > m ? b : m;
    }
    return m < P.phib[0] ? 0 : (m < P.phib[1] ? 1 : (m < P.phib[2] ? 2 : 3));
}
__device__ __forceinline__ int branch_of(const DevParams& P, const float* ph) {
    float m = ph[0];
#pragma unroll
    for (int o = 1; o < 6; o++) m = fmaxf(m, ph[o]);
    const Cst<float>& K = P.cf;
    int br = m < K.phi1 ? 0 : (m < K.phi2 ? 1 : (m < K.phi3 ? 2 : 3));
    return m != m ? 3 : br;
}

// a + b + c with error-free transformations (Knuth's TwoSum): s + e is the exact sum of the
// three, returned rounded once. For FP32 operands; the FP64 form never calls it.
__device__ __forceinline__ float two_sum(float a, float b, float& e) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return s;
}
__device__ __forceinline__ float sum3_compensated(float a, float b, float c) {
    float e1, e2;
    const float s1 = two_sum(a, b, e1);
    const float s2 = two_sum(s1, c, e2);
    return __fadd_rn(s2, __fadd_rn(e1, e2));
}

template <int DIR, int TL, int TC, int NTHREADS, class R, class CellFn, class FidxFn>
__device__ __forceinline__ void sweep_epilogue(const SweepArgs& a, const R* sF, int c0, int l0, int other, int nc,
                                               int nl, const CellFn& cell, const FidxFn& fidx) {
    constexpr int NF = TC + 1;
    const DevParams& P = a.P;
    const long long pl = P.plane;
    // cells t = 0..nc-1 (full position c0 + t + NG)
    const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
    const long long vplane = (long long)vxt * vyt * vzt;
    R* acc = static_cast<R*>(a.acc);
    const R* Fvr = static_cast<const R*>(a.Fv);
    for (int it = threadIdx.x; it < TL * TC; it += NTHREADS) {
        int l, t;
        if (DIR == 0) { l = it / TC; t = it - l * TC; } else { t = it / TL; l = it - t * TL; }
        if (l >= nl || t >= nc) continue;
        const long long c = cell(l, c0 + t + NG);
        R d[5];
#pragma unroll
        for (int n = 0; n < 5; n++) d[n] = sF[n * TL * NF + fidx(l, t)] - sF[n * TL * NF + fidx(l, t + 1)];
        if (Fvr) {
            // Fv index = full index - 2 in every dimension (viscous.jl:119, div.jl:14-39)
            long long vi, vj, vk;
            const int g = c0 + t + NG - 2;
            if (DIR == 0) { vi = g; vj = l0 + l + NG - 2; vk = other + NG - 2; }
            else if (DIR == 1) { vi = l0 + l + NG - 2; vj = g; vk = other + NG - 2; }
            else { vi = l0 + l + NG - 2; vj = other + NG - 2; vk = g; }
            const long long vc = vi + (long long)vxt * (vj + (long long)vyt * vk);
            const long long vs = DIR == 0 ? 1 : (DIR == 1 ? (long long)vxt : (long long)vxt * vyt);
            const R k1 = R(1) / R(12), k2 = R(-2) / R(3);
#pragma unroll
            for (int n = 0; n < 4; n++) {
                const R* F = Fvr + n * vplane + vc;
                d[n + 1] += k1 * (F[-2 * vs] - F[2 * vs]) + k2 * (F[-vs] - F[vs]);
            }
        }
        if constexpr (sizeof(R) == 4) {
            if (a.J32 && (a.out_mode == OUT_RHS || a.out_mode == OUT_STAGE)) {
                // F3D_PREC_REF32: Float32 result, J dt L added to U and combined in Float32
                // (div.jl:40-48, utils.jl:57-70)
                if (a.out_mode == OUT_RHS) {
                    const float Jc = a.J32[c];
#pragma unroll
                    for (int n = 0; n < 5; n++) a.out32[c + n * pl] = (acc[c + n * pl] + d[n]) * Jc;
                } else {
                    const float Jact = a.J32[c] * a.dt32;
#pragma unroll
                    for (int n = 0; n < 5; n++) {
                        const float u = a.U32[c + n * pl];
                        if (a.stage1_copy) a.Un32[c + n * pl] = u;
                        float un = u + (acc[c + n * pl] + d[n]) * Jact;
                        if (a.combine) un = un * a.ca32 + a.Un32[c + n * pl] * a.cb32;
                        a.U32[c + n * pl] = un;
                    }
                }
                continue;
            }
        }
        // sum of the three directions: in the arithmetic type, or (mixed form, acc2 set) the xi
        // and eta sweeps' FP32 differences and this sweep's summed with compensation, so the
        // result is the exact sum rounded once to FP32 (relative to the sum, not to the terms
        // that cancel in it)
        auto total = [&](int n) -> double {
            if constexpr (sizeof(R) == 4) {
                if (a.acc2) return to_f64(sum3_compensated(acc[c + n * pl], a.acc2[c + n * pl], d[n]));
            }
            return to_f64(acc[c + n * pl] + d[n]);
        };
        if (a.out_mode == OUT_SET) {
#pragma unroll
            for (int n = 0; n < 5; n++) acc[c + n * pl] = d[n];
        } else if (a.out_mode == OUT_ADD) {
#pragma unroll
            for (int n = 0; n < 5; n++) acc[c + n * pl] += d[n];
        } else if (a.out_mode == OUT_RHS) {
            const double Jc = a.J[c];
#pragma unroll
            for (int n = 0; n < 5; n++) a.out[c + n * pl] = Jc * total(n);
        } else {  // OUT_STAGE: RK state accumulation in FP64
            const double Jact = a.J[c] * (a.dtl ? a.dtl[c] : a.dt);  // div_LTS: per-cell dt
#pragma unroll
            for (int n = 0; n < 5; n++) {
                const double u = a.U[c + n * pl];
                if (a.stage1_copy) a.Un[c + n * pl] = u;
                double un = u + total(n) * Jact;
                if (a.combine) un = un * a.ca + a.Un[c + n * pl] * a.cb;
                a.U[c + n * pl] = un;
            }
        }
    }
}

}  // namespace f3d
