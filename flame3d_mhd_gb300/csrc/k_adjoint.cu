// k_adjoint.cu — discrete adjoint (VJP) of the FP64 right-hand side.
//
// Forward chain of one RHS:  U --c2Prim--> Q (interior) --ghost fill--> Q (all cells)
//   --split--> Fp, Fm --reconstruction--> face fluxes --difference x J--> L,
//   plus Q --gradients--> Fv --CD4 x J--> L (viscous).
// The kernels below run it backwards for a cotangent Lb of L (interior cells):
//   k_sweep_vjp<d,char> face cotangents from J Lb, reverse of UP7/WENO7/WENO5/NND2 on the
//                       forward branch (component- or characteristic-wise: char_face_vjp),
//                       reverse of the split (SW, LF, VL, AUSM), into Qb;
//   k_visc_fvb          Fv cotangents: transpose of the CD4 divergence (div.jl:14-48);
//   k_visc_vjp          reverse of viscousFlux per cell into gradient/centre cotangents;
//   k_visc_gather       transpose of the CD4 gradients (viscous.jl:29-42) into Qb;
//   k_fill_vjp          transpose of the ghost rules: ghost Qb to its interior source;
//   k_c2prim_vjp        reverse of c2Prim into Ub, fused with out = beta out + alpha Ub.
// Contributions that cross tile boundaries are added with FP64 atomics, so gradients are
// accurate but their last bits depend on the order of those additions.
#include "f3d_adjoint.cuh"
#include "f3d_kernels.cuh"

namespace f3d {

// Tile of TL lines x TC cells; NT threads cover the TL x (TC + 8) stencil positions of
// phases A and C. About 140 registers a thread (component-wise) and 59.5 KB of shared
// memory a block for 4-line tiles (the split fluxes, their cotangents, the sensor and the UP7
// face cotangents gathered in Phase C): three blocks per SM.
#ifndef V_TL0
#define V_TL0 4
#define V_NT0 96
#define V_MB0 3
#define V_TL12 4
#define V_NT12 96
#define V_MB12 3
#endif
// characteristic-wise reverse sweeps: the reverse of a characteristic WENO face holds more
// state (its eigenvectors, a side's stencil of one field and its cotangents). Smaller blocks
// (xi 4 x 64 on 64 threads, three per SM; eta / zeta 4 x 64 on 96 threads, two per SM):
// adjoint / forward 3.70 on the 256x64x64 shock tube against 3.78 for the component-wise
// shape and 3.90 for 192-thread blocks with 255 registers (same box, alternating builds)
#ifndef V_C_TL0
#define V_C_TL0 4
#define V_C_NT0 64
#define V_C_MB0 3
#define V_C_TL12 4
#define V_C_NT12 96
#define V_C_MB12 2
#endif
template <int DIR, bool CHAR = false> struct VTile;
template <> struct VTile<0, false> { static constexpr int TL = V_TL0, TC = 64, NT = V_NT0, MINB = V_MB0; };
template <> struct VTile<1, false> { static constexpr int TL = V_TL12, TC = 64, NT = V_NT12, MINB = V_MB12; };
template <> struct VTile<2, false> { static constexpr int TL = V_TL12, TC = 64, NT = V_NT12, MINB = V_MB12; };
template <> struct VTile<0, true> { static constexpr int TL = V_C_TL0, TC = 64, NT = V_C_NT0, MINB = V_C_MB0; };
template <> struct VTile<1, true> { static constexpr int TL = V_C_TL12, TC = 64, NT = V_C_NT12, MINB = V_C_MB12; };
template <> struct VTile<2, true> { static constexpr int TL = V_C_TL12, TC = 64, NT = V_C_NT12, MINB = V_C_MB12; };

template <int DIR, bool CHAR> constexpr size_t vjp_smem_bytes() {
    using T = VTile<DIR, CHAR>;
    return sizeof(double) * ((size_t)T::TL * (T::TC + 8) * 21 + 5 * (size_t)T::TL * (T::TC + 1)) +
           sizeof(int) * (2 * (size_t)T::TL * (T::TC + 1) + 4);
}

template <int DIR, bool CHAR>
__global__ void __launch_bounds__(VTile<DIR, CHAR>::NT, VTile<DIR, CHAR>::MINB) k_sweep_vjp(const AdjArgs a) {
    constexpr int TL = VTile<DIR, CHAR>::TL, TC = VTile<DIR, CHAR>::TC, NP = TC + 8, NT = VTile<DIR, CHAR>::NT;
    const DevParams& P = a.P;
    const bool hybrid = P.fixed_branch < 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sFp = reinterpret_cast<double*>(smem_raw);
    double* sFm = sFp + 5 * TL * NP;
    double* sFpb = sFm + 5 * TL * NP;
    double* sFmb = sFpb + 5 * TL * NP;
    double* sPhi = sFmb + 5 * TL * NP;
    // cotangents of the UP7 faces (zero elsewhere): UP7 is linear, so its transpose is applied
    // as a gather in Phase C (each stencil position sums its seven faces) instead of 70
    // shared-memory atomics per face
    double* sG = sPhi + TL * NP;
    constexpr int NFV = TC + 1;
    auto gidx = [&](int l, int t) { return DIR == 0 ? l * NFV + t : t * TL + l; };

    const int Nd = DIR == 0 ? P.nx : (DIR == 1 ? P.ny : P.nz);
    const int Nl = DIR == 0 ? P.ny : P.nx;
    int c0, l0, other;
    if (DIR == 0) { c0 = blockIdx.x * TC; l0 = blockIdx.y * TL; other = blockIdx.z; }
    else { l0 = blockIdx.x * TL; c0 = blockIdx.y * TC; other = blockIdx.z; }
    const int nc = min(TC, Nd - c0);
    const int nl = min(TL, Nl - l0);
    const bool last_tile = c0 + nc == Nd;
    const int nfaces = nc + (last_tile ? 1 : 0);  // faces c0..c0+nc-1, plus face N on the last tile
    const long long stride = DIR == 0 ? 1 : (DIR == 1 ? (long long)P.nxt : (long long)P.nxt * P.nyt);
    auto cell = [&](int l, int g) -> long long {
        if (DIR == 0) return lin3(P, g, l0 + l + NG, other + NG);
        if (DIR == 1) return lin3(P, l0 + l + NG, g, other + NG);
        return lin3(P, l0 + l + NG, other + NG, g);
    };
    auto sidx = [&](int l, int p) { return DIR == 0 ? l * NP + p : p * TL + l; };
    const long long pl = P.plane;

    int* list7 = reinterpret_cast<int*>(sG + 5 * TL * NFV);
    int* list5 = list7 + TL * (TC + 1);
    int* counts = list5 + TL * (TC + 1);
    if (threadIdx.x < 2) counts[threadIdx.x] = 0;
    for (int it = threadIdx.x; it < 5 * TL * NFV; it += NT) sG[it] = 0.0;
    // Phase A: forward split at positions 0..nc+7 (full index c0 + p); zero the cotangents
    for (int it = threadIdx.x; it < TL * NP; it += NT) {
        int l, p;
        if (DIR == 0) { l = it / NP; p = it - l * NP; } else { p = it / TL; l = it - p * TL; }
        const int s = sidx(l, p);
        for (int n = 0; n < 5; n++) {
            sFpb[n * TL * NP + s] = 0.0;
            sFmb[n * TL * NP + s] = 0.0;
        }
        if (l >= nl || p >= nc + 8) continue;
        const long long c = cell(l, c0 + p);
        double q[6], fp[5], fm[5];
        for (int n = 0; n < 6; n++) q[n] = a.Q[c + n * pl];
        split_cell<double>(P.split, P.cd, q, a.csnd[c], a.A[0][c], a.A[1][c], a.A[2][c], a.Ah[0][c], a.Ah[1][c],
                           a.Ah[2][c], a.S[c], fp, fm);
        for (int n = 0; n < 5; n++) {
            sFp[n * TL * NP + s] = fp[n];
            sFm[n * TL * NP + s] = fm[n];
        }
        if (hybrid) sPhi[s] = a.phi[c];
    }
    __syncthreads();

    // Phase B: owned faces t (interior face c0+t, between positions t+3 and t+4). UP7 and
    // NND2 faces at once; WENO7 / WENO5 faces queued and done by consecutive threads.
    auto face_vjp = [&](int l, int t, int br) {
        const int f = c0 + t;  // interior face index 0..Nd
        // L_c = J_c (F[left face of c] - F[right face of c]): face f is the left face of
        // interior cell f and the right face of interior cell f-1
        double Fb[5] = {0, 0, 0, 0, 0};
        const long long cr = cell(l, f + NG), cl = cr - stride;
        if (f < Nd) {
            const double j = a.J[cr];
            for (int n = 0; n < 5; n++) Fb[n] += j * a.Lb[cr + n * pl];
        }
        if (f >= 1) {
            const double j = a.J[cl];
            for (int n = 0; n < 5; n++) Fb[n] -= j * a.Lb[cl + n * pl];
        }
        if (br == 0) {  // UP7 (schemes.jl:119-142): the face cotangent, gathered in Phase C
            for (int n = 0; n < 5; n++) sG[n * TL * NFV + gidx(l, t)] = Fb[n];
            return;
        }
        const double s0 = (br == 1 || br == 2) ? 2.0 / (a.S[cl] + a.S[cr]) : 0.0;
        double s0b_ = 0.0;
        double* s0b = a.mb[0] ? &s0b_ : nullptr;  // metric cotangent wanted
        if (CHAR && (br == 1 || br == 2)) {
            // characteristic-wise WENO: the face state is the mean of the two cells beside it
            const double st[7] = {0.5 * (a.Q[cr + pl] + a.Q[cl + pl]), 0.5 * (a.Q[cr + 2 * pl] + a.Q[cl + 2 * pl]),
                                  0.5 * (a.Q[cr + 3 * pl] + a.Q[cl + 3 * pl]), 0.5 * (a.Q[cr + 5 * pl] + a.Q[cl + 5 * pl]),
                                  (a.A[0][cr] + a.A[0][cl]) * 0.5, (a.A[1][cr] + a.A[1][cl]) * 0.5,
                                  (a.A[2][cr] + a.A[2][cl]) * 0.5};
            double stb[7] = {0, 0, 0, 0, 0, 0, 0};
            auto FPv = [&](int n, int pos) { return sFp[n * TL * NP + sidx(l, pos)]; };
            auto FMv = [&](int n, int pos) { return sFm[n * TL * NP + sidx(l, pos)]; };
            auto addP = [&](int n, int pos, double v) { atomicAdd(&sFpb[n * TL * NP + sidx(l, pos)], v); };
            auto addM = [&](int n, int pos, double v) { atomicAdd(&sFmb[n * TL * NP + sidx(l, pos)], v); };
            char_face_vjp(P, br, t, s0, st, Fb, FPv, FMv, addP, addM, stb, s0b);
            const int qv[4] = {1, 2, 3, 5};  // u, v, w, T
            for (int k = 0; k < 4; k++) {
                const double h = 0.5 * stb[k];
                if (h != 0.0) {
                    atomicAdd(&a.Qb[cl + qv[k] * pl], h);
                    atomicAdd(&a.Qb[cr + qv[k] * pl], h);
                }
            }
            if (a.mb[0])
                for (int j = 0; j < 3; j++) {
                    const double h = 0.5 * a.mscale * stb[4 + j];
                    atomicAdd(&a.mb[j][cl], h);
                    atomicAdd(&a.mb[j][cr], h);
                }
        }
        for (int n = 0; n < 5 && !(CHAR && (br == 1 || br == 2)); n++) {
            const double g = Fb[n];
            if (g == 0.0) continue;
            double* pb = sFpb + n * TL * NP;
            double* mb = sFmb + n * TL * NP;
            const double* vp = sFp + n * TL * NP;
            const double* vm = sFm + n * TL * NP;
            auto P_ = [&](int pos) { return vp[sidx(l, pos)]; };
            auto M_ = [&](int pos) { return vm[sidx(l, pos)]; };
            if (br == 1) {  // WENO7, (fp + fm)/12
                double V[7], Vb[7];
                for (int k = 0; k < 7; k++) V[k] = P_(t + k);
                weno7_vjp(V, s0, g * (1.0 / 12.0), Vb, s0b);
                for (int k = 0; k < 7; k++) atomicAdd(&pb[sidx(l, t + k)], Vb[k]);
                for (int k = 0; k < 7; k++) V[k] = M_(t + 7 - k);
                weno7_vjp(V, s0, g * (1.0 / 12.0), Vb, s0b);
                for (int k = 0; k < 7; k++) atomicAdd(&mb[sidx(l, t + 7 - k)], Vb[k]);
            } else if (br == 2) {  // WENO5, (fp + fm)/6: Fp at t+1..t+5, Fm at t+6..t+2
                double V[5], Vb[5];
                for (int k = 0; k < 5; k++) V[k] = P_(t + 1 + k);
                weno5_vjp(V, s0, g * (1.0 / 6.0), Vb, s0b);
                for (int k = 0; k < 5; k++) atomicAdd(&pb[sidx(l, t + 1 + k)], Vb[k]);
                for (int k = 0; k < 5; k++) V[k] = M_(t + 6 - k);
                weno5_vjp(V, s0, g * (1.0 / 6.0), Vb, s0b);
                for (int k = 0; k < 5; k++) atomicAdd(&mb[sidx(l, t + 6 - k)], Vb[k]);
            } else {  // NND2 (schemes.jl:277-286): minmod picks one difference or none
                // fp = Fp[t+3] + 0.5 minmod(Fp[t+4]-Fp[t+3], Fp[t+3]-Fp[t+2])
                const double a1 = P_(t + 4) - P_(t + 3), b1 = P_(t + 3) - P_(t + 2);
                atomicAdd(&pb[sidx(l, t + 3)], g);
                if (a1 * b1 > 0.0) {
                    if (fabs(a1) > fabs(b1)) {
                        atomicAdd(&pb[sidx(l, t + 3)], 0.5 * g);
                        atomicAdd(&pb[sidx(l, t + 2)], -0.5 * g);
                    } else {
                        atomicAdd(&pb[sidx(l, t + 4)], 0.5 * g);
                        atomicAdd(&pb[sidx(l, t + 3)], -0.5 * g);
                    }
                }
                // fm = Fm[t+4] - 0.5 minmod(Fm[t+5]-Fm[t+4], Fm[t+4]-Fm[t+3])
                const double a2 = M_(t + 5) - M_(t + 4), b2 = M_(t + 4) - M_(t + 3);
                atomicAdd(&mb[sidx(l, t + 4)], g);
                if (a2 * b2 > 0.0) {
                    if (fabs(a2) > fabs(b2)) {
                        atomicAdd(&mb[sidx(l, t + 4)], -0.5 * g);
                        atomicAdd(&mb[sidx(l, t + 3)], 0.5 * g);
                    } else {
                        atomicAdd(&mb[sidx(l, t + 5)], -0.5 * g);
                        atomicAdd(&mb[sidx(l, t + 4)], 0.5 * g);
                    }
                }
            }
        }
        if (s0b && s0b_ != 0.0) {
            // s0 = 2 / (S_l + S_r): both |A| get -s0^2/2 s0-bar, and |A| passes A_j / |A| to A_j
            const double Sb = -0.5 * s0 * s0 * s0b_ * a.mscale;
            const long long cc[2] = {cl, cr};
            for (int e = 0; e < 2; e++) {
                const double r = Sb / a.S[cc[e]];
                for (int j = 0; j < 3; j++) atomicAdd(&a.mb[j][cc[e]], r * a.A[j][cc[e]]);
            }
        }
    };
    for (int it = threadIdx.x; it < TL * (TC + 1); it += NT) {
        int l, t;
        if (DIR == 0) { l = it / (TC + 1); t = it - l * (TC + 1); } else { t = it / TL; l = it - t * TL; }
        if (l >= nl || t >= nfaces) continue;
        int br = P.fixed_branch;
        if (hybrid) {
            unsigned long long m = __double_as_longlong(sPhi[sidx(l, t + 1)]);
            for (int o = 2; o <= 6; o++) {
                unsigned long long b = __double_as_longlong(sPhi[sidx(l, t + o)]);
                m = b > m ? b : m;
            }
            br = m < P.phib[0] ? 0 : (m < P.phib[1] ? 1 : (m < P.phib[2] ? 2 : 3));
            if (br == 1 || br == 2) {
                const int k = atomicAdd(&counts[br - 1], 1);
                (br == 1 ? list7 : list5)[k] = it;
                continue;
            }
        }
        face_vjp(l, t, br);
    }
    if (hybrid) {
        __syncthreads();
        const int n7 = counts[0], n5 = counts[1];
        for (int k = threadIdx.x; k < n7 + n5; k += NT) {
            const int it = k < n7 ? list7[k] : list5[k - n7];
            int l, t;
            if (DIR == 0) { l = it / (TC + 1); t = it - l * (TC + 1); } else { t = it / TL; l = it - t * TL; }
            face_vjp(l, t, k < n7 ? 1 : 2);
        }
    }
    __syncthreads();

    // Phase C: reverse of the split at every position, into Qb
    for (int it = threadIdx.x; it < TL * NP; it += NT) {
        int l, p;
        if (DIR == 0) { l = it / NP; p = it - l * NP; } else { p = it / TL; l = it - p * TL; }
        if (l >= nl || p >= nc + 8) continue;
        const int s = sidx(l, p);
        double fpb[5], fmb[5];
        bool any = false;
        for (int n = 0; n < 5; n++) {
            // UP7 faces t = p - k take Fp here with coefficient lin[k], faces t = p - 7 + k
            // take Fm here with lin[k] (positions t..t+6 and t+7..t+1 of face t)
            const double* G = sG + n * TL * NFV;
            double gp = 0.0, gm = 0.0;
#pragma unroll
            for (int k = 0; k < 7; k++) {
                const int tp = p - k, tm = p - 7 + k;
                if (tp >= 0 && tp < NFV) gp += P.cd.lin[k] * G[gidx(l, tp)];
                if (tm >= 0 && tm < NFV) gm += P.cd.lin[k] * G[gidx(l, tm)];
            }
            fpb[n] = sFpb[n * TL * NP + s] + gp;
            fmb[n] = sFmb[n * TL * NP + s] + gm;
            any |= fpb[n] != 0.0 || fmb[n] != 0.0;
        }
        if (!any) continue;
        const long long c = cell(l, c0 + p);
        double q[6], qb[6] = {0, 0, 0, 0, 0, 0};
        double mg[7] = {0, 0, 0, 0, 0, 0, 0};
        double* mgp = a.mb[0] ? mg : nullptr;
        for (int n = 0; n < 6; n++) q[n] = a.Q[c + n * pl];
        const double A3[3] = {a.A[0][c], a.A[1][c], a.A[2][c]};
        const double S = a.S[c];
        if (P.split == F3D_SPLIT_SW)
            split_sw_vjp(P.cd, q, a.csnd[c], A3[0], A3[1], A3[2], a.Ah[0][c], a.Ah[1][c], a.Ah[2][c], S, fpb, fmb, qb,
                         mgp);
        else if (P.split == F3D_SPLIT_LF)
            split_lf_vjp(P.cd, q, a.csnd[c], A3[0], A3[1], A3[2], S, fpb, fmb, qb, mgp);
        else  // van Leer, AUSM
            split_mach_vjp(P.split, P.cd, q, a.csnd[c], A3[0], A3[1], A3[2], S, fpb, fmb, qb, mgp);
        for (int n = 0; n < 6; n++)
            if (qb[n] != 0.0) atomicAdd(&a.Qb[c + n * pl], qb[n]);
        if (mgp) {
            // A/|A| and |A| derive from A: A_j-bar += H_j-bar/S - (H-bar . A) A_j/S^3 + S-bar A_j/S
            const double iS = 1.0 / S;
            const double hA = (mg[3] * A3[0] + mg[4] * A3[1] + mg[5] * A3[2]) * iS * iS * iS;
            for (int j = 0; j < 3; j++) {
                const double b = mg[j] + mg[3 + j] * iS - hA * A3[j] + mg[6] * A3[j] * iS;
                if (b != 0.0) atomicAdd(&a.mb[j][c], a.mscale * b);
            }
        }
    }
}

// ---- viscous ---------------------------------------------------------------------------
// Fv_d cotangents at box cells: the divergence adds, for interior cell c,
// J_c [k1 (F[c-2] - F[c+2]) + k2 (F[c-1] - F[c+1])] to momentum/energy (div.jl:14-48).
__global__ void k_visc_fvb(const DevParams P, const double* __restrict__ Lb, const double* __restrict__ J,
                           double* Fvbx, double* Fvby, double* Fvbz) {
    const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
    const long long vpl = (long long)vxt * vyt * vzt;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= vpl) return;
    int vi, vj, vk;
    split3(t, P.dvxt, P.dvyt, vi, vj, vk);
    const int gi = vi + 2, gj = vj + 2, gk = vk + 2;  // full cell index
    const double k1 = 1.0 / 12.0, k2 = -2.0 / 3.0;
    const int g[3] = {gi, gj, gk};
    const int N[3] = {P.nx, P.ny, P.nz};
    const long long st[3] = {1, (long long)P.nxt, (long long)P.nxt * P.nyt};
    double* out[3] = {Fvbx, Fvby, Fvbz};
    const long long c = lin3(P, gi, gj, gk);
    auto inside = [&](int d, int idx) { return idx >= NG && idx < N[d] + NG; };
    for (int d = 0; d < 3; d++) {
        // transverse indices must be interior for any interior cell to use this Fv_d value
        bool tr = true;
        for (int e = 0; e < 3; e++)
            if (e != d && !inside(e, g[e])) tr = false;
        double acc[4] = {0, 0, 0, 0};
        if (tr) {
            const int offs[4] = {2, -2, 1, -1};
            const double coef[4] = {k1, -k1, k2, -k2};  // F[c'] enters cell c'+2 with +k1, c'-2 with -k1, ...
            for (int o = 0; o < 4; o++) {
                const int gg = g[d] + offs[o];
                if (!inside(d, gg)) continue;
                const long long cc = c + offs[o] * st[d];
                const double w = coef[o] * J[cc];
                for (int n = 0; n < 4; n++) acc[n] += w * Lb[cc + (n + 1) * P.plane];
            }
        }
        for (int n = 0; n < 4; n++) out[d][t + n * vpl] = acc[n];
    }
}

// Reverse of viscousFlux at one box cell (viscous.jl:10-64, 107-133): Fv cotangents into
// cotangents of the 12 computational gradients (xi, eta, zeta of u, v, w, T), stored
// in gb (12 x box), and of the centre values u, v, w, T (added to Qb directly).
__global__ void k_visc_vjp(const DevParams P, const double* __restrict__ Q, const double* m0, const double* m1,
                           const double* m2, const double* m3, const double* m4, const double* m5, const double* m6,
                           const double* m7, const double* m8, const double* __restrict__ J, const double* Fvbx,
                           const double* Fvby, const double* Fvbz, double* gb, double* Qb, MetricBar mbar) {
    const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
    const long long vpl = (long long)vxt * vyt * vzt;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= vpl) return;
    int vi, vj, vk;
    split3(t, P.dvxt, P.dvyt, vi, vj, vk);
    const long long c = lin3(P, vi + 2, vj + 2, vk + 2);
    const long long pl = P.plane, sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const double M[3][3] = {{m0[c], m1[c], m2[c]}, {m3[c], m4[c], m5[c]}, {m6[c], m7[c], m8[c]}};  // M[d][x]
    const double Jac = J[c];
    const double T = Q[c + 5 * pl];
    const double sT = sqrt(T);
    const double rTs = 1.0 / (T + P.t_s);
    const double mu = P.c_s * T * sT * rTs;
    const double lam = mu * P.cd.cp_pr;
    const double c1 = 1.0 / 12.0, c2 = -2.0 / 3.0, c23 = 2.0 / 3.0;
    // forward: computational gradients G[var][d] of (u, v, w, T) and physical D[var][x]
    const int vars[4] = {1, 2, 3, 5};
    const long long st[3] = {1, sy, sz};
    double G[4][3], D[4][3];
    for (int a = 0; a < 4; a++)
        for (int d = 0; d < 3; d++) {
            const double* f = Q + vars[a] * pl + c;
            G[a][d] = c1 * (f[-2 * st[d]] - f[2 * st[d]]) + c2 * (f[-st[d]] - f[st[d]]);
        }
    for (int a = 0; a < 4; a++)
        for (int x = 0; x < 3; x++) D[a][x] = (G[a][0] * M[0][x] + G[a][1] * M[1][x] + G[a][2] * M[2][x]) * Jac;
    const double uvw[3] = {Q[c + pl], Q[c + 2 * pl], Q[c + 3 * pl]};
    const double dv = D[0][0] + D[1][1] + D[2][2];
    double tau[3][3];
    for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++) tau[x][y] = mu * (D[x][y] + D[y][x]);
    for (int x = 0; x < 3; x++) tau[x][x] = mu * (2.0 * D[x][x] - c23 * dv);
    // E_x = sum_y u_y tau[y][x] + lam dT/dx
    // reverse: Fv_d[n] = sum_x M[d][x] tau[x][n] (n < 3), Fv_d[3] = sum_x M[d][x] E_x
    const double* Fvb[3] = {Fvbx, Fvby, Fvbz};
    double taub[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}}, Eb[3] = {0, 0, 0};
    for (int d = 0; d < 3; d++) {
        const double fb[4] = {Fvb[d][t], Fvb[d][t + vpl], Fvb[d][t + 2 * vpl], Fvb[d][t + 3 * vpl]};
        for (int x = 0; x < 3; x++) {
            for (int n = 0; n < 3; n++) taub[x][n] += M[d][x] * fb[n];
            Eb[x] += M[d][x] * fb[3];
        }
    }
    double ub[3] = {0, 0, 0}, lamb = 0, mub = 0;
    double Db[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int x = 0; x < 3; x++) {
        for (int y = 0; y < 3; y++) {
            ub[y] += Eb[x] * tau[y][x];
            taub[y][x] += Eb[x] * uvw[y];
        }
        lamb += Eb[x] * D[3][x];
        Db[3][x] += Eb[x] * lam;
    }
    // tau is symmetric in the forward; taub holds the cotangent of each (x,y) entry as used
    double dvb = 0;
    for (int x = 0; x < 3; x++)
        for (int y = 0; y < 3; y++) {
            const double g = taub[x][y];
            if (x == y) {
                mub += g * (2.0 * D[x][x] - c23 * dv);
                Db[x][x] += g * mu * 2.0;
                dvb += -g * mu * c23;
            } else {
                mub += g * (D[x][y] + D[y][x]);
                Db[x][y] += g * mu;
                Db[y][x] += g * mu;
            }
        }
    Db[0][0] += dvb;
    Db[1][1] += dvb;
    Db[2][2] += dvb;
    // lambda = cp mu / Pr; mu = C_s T^1.5 / (T + T_s)
    mub += lamb * P.cd.cp_pr;
    const double Tb_mu = mub * P.c_s * (1.5 * sT * (T + P.t_s) - T * sT) * (rTs * rTs);
    // D[a][x] = (sum_d G[a][d] M[d][x]) J
    for (int a = 0; a < 4; a++)
        for (int d = 0; d < 3; d++) {
            double g = 0;
            for (int x = 0; x < 3; x++) g += Db[a][x] * M[d][x];
            gb[t + (a * 3 + d) * vpl] = g * Jac;
        }
    atomicAdd(&Qb[c + pl], ub[0]);
    atomicAdd(&Qb[c + 2 * pl], ub[1]);
    atomicAdd(&Qb[c + 3 * pl], ub[2]);
    atomicAdd(&Qb[c + 5 * pl], Tb_mu);
    if (mbar.m[0]) {
        // metric cotangents of this cell: the projections Fv_d = sum_x M[d][x] (tau, E)[x] and
        // the gradients D[a][x] = (sum_d G[a][d] M[d][x]) J
        double E[3];
        for (int x = 0; x < 3; x++) E[x] = uvw[0] * tau[0][x] + uvw[1] * tau[1][x] + uvw[2] * tau[2][x] + lam * D[3][x];
        double Jb = 0.0;
        for (int a = 0; a < 4; a++)
            for (int x = 0; x < 3; x++) Jb += Db[a][x] * D[a][x];
        for (int d = 0; d < 3; d++) {
            const double fb[4] = {Fvb[d][t], Fvb[d][t + vpl], Fvb[d][t + 2 * vpl], Fvb[d][t + 3 * vpl]};
            for (int x = 0; x < 3; x++) {
                double b = fb[0] * tau[x][0] + fb[1] * tau[x][1] + fb[2] * tau[x][2] + fb[3] * E[x];
                for (int a = 0; a < 4; a++) b += Db[a][x] * G[a][d] * Jac;
                mbar.m[3 * d + x][c] += mbar.scale * b;  // one thread per cell, after the sweeps
            }
        }
        mbar.J[c] += mbar.scale * Jb / Jac;
    }
}

// J-bar += scale sum_n Lb L / J at interior cells (L = J D: the direct dependence on J)
__global__ void k_jbar(const DevParams P, const double* __restrict__ Lb, const double* __restrict__ L,
                       const double* __restrict__ J, double* Jbar, double scale) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.nx * P.ny * P.nz) return;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    const long long c = lin3(P, i + NG, j + NG, k + NG), pl = P.plane;
    double s = 0.0;
    for (int n = 0; n < 5; n++) s += Lb[c + n * pl] * L[c + n * pl];
    Jbar[c] += scale * s / J[c];
}

// Transpose of the CD4 gradients: G[c'] = c1 (f[c'-2] - f[c'+2]) + c2 (f[c'-1] - f[c'+1]),
// gathered at every cell c from the box cells c' = c -+ 1, 2 that used it.
__global__ void k_visc_gather(const DevParams P, const double* __restrict__ gb, double* Qb) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
    const long long vpl = (long long)vxt * vyt * vzt;
    const double c1 = 1.0 / 12.0, c2 = -2.0 / 3.0;
    const int g[3] = {i, j, k};
    const int vn[3] = {vxt, vyt, vzt};
    const int vars[4] = {1, 2, 3, 5};
    double acc[4] = {0, 0, 0, 0};
    for (int d = 0; d < 3; d++) {
        // box index of c along the other dimensions must be valid
        bool ok = true;
        int vb[3];
        for (int e = 0; e < 3; e++) {
            vb[e] = g[e] - 2;
            if (e != d && (vb[e] < 0 || vb[e] >= vn[e])) ok = false;
        }
        if (!ok) continue;
        // c = c' - 2 gets +c1, c = c' + 2 gets -c1, c = c' - 1 gets +c2, c = c' + 1 gets -c2
        const int offs[4] = {2, -2, 1, -1};
        const double coef[4] = {c1, -c1, c2, -c2};
        for (int o = 0; o < 4; o++) {
            int vv[3] = {vb[0], vb[1], vb[2]};
            vv[d] += offs[o];
            if (vv[d] < 0 || vv[d] >= vn[d]) continue;
            const long long tc = vv[0] + (long long)vxt * (vv[1] + (long long)vyt * vv[2]);
            for (int a = 0; a < 4; a++) acc[a] += coef[o] * gb[tc + (a * 3 + d) * vpl];
        }
    }
    for (int a = 0; a < 4; a++)
        if (acc[a] != 0.0) Qb[c + vars[a] * P.plane] += acc[a];
}

// ---- ghost fill and c2Prim -----------------------------------------------------------
// Transpose of the composed ghost rules: a ghost cell's cotangent goes to its interior
// source (copies and mirrors), nowhere for Dirichlet values; isothermal walls pass p, T
// through T_g = 2 T_w - T_s and rho_g = p_s / (Rg T_g).
// Inflow-profile cotangents (when a buffer is set) receive pscale times theirs: the RHS VJP
// scales its state cotangent by alpha after c2Prim, and the profile enters before it.
__global__ void k_fill_vjp(const DevParams P, const double* __restrict__ Q, double* Qb, double pscale) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    if (i >= NG && i < P.nx + NG && j >= NG && j < P.ny + NG && k >= NG && k < P.nz + NG) return;
    const GhostChain ch = resolve_ghost(P, i, j, k);
    const bool to_profile = ch.dirichlet >= 0 && P.bc[ch.dirichlet].kind == F3D_BC_INFLOW_PROFILE &&
                            P.profb[ch.dirichlet] != nullptr;
    if (ch.dirichlet >= 0 && !to_profile) return;  // a fixed state: no dependence
    const long long pl = P.plane;
    double gq[6];
    for (int n = 0; n < 6; n++) gq[n] = Qb[c + n * pl];
    const long long s = to_profile ? 0 : lin3(P, ch.si, ch.sj, ch.sk);
    double sq_[6] = {gq[0], gq[1], gq[2], gq[3], gq[4], gq[5]};
    if (ch.nmirror & 1) {
        sq_[1] = -gq[1];
        sq_[2] = -gq[2];
        sq_[3] = -gq[3];
    }
    if (ch.iso_face >= 0) {
        // forward: Tg = 2 Tw - Ts, rho_g = p / (Rg Tg) with p the source pressure
        const double Tg = Q[c + 5 * pl], pg = Q[c + 4 * pl];
        const double rhob = gq[0];
        sq_[0] = 0.0;
        sq_[4] = gq[4] + rhob / (P.rg * Tg);
        const double Tgb = gq[5] - rhob * pg / (P.rg * Tg * Tg);
        sq_[5] = -Tgb;
    }
    if (to_profile) {
        // the chain's first value is the profile state q = (rho, u, v, w, p, p / (rho Rg)) of
        // its transverse point: pass the cotangent to (rho, u, v, w, p) of that point
        const double* pr = P.prof[ch.dirichlet] + ch.poff;
        double* pb = P.profb[ch.dirichlet] + ch.poff;
        const double rho = pr[0], p = pr[4 * ch.pst];
        const double T = p / (rho * P.rg);
        const double b[5] = {sq_[0] - sq_[5] * T / rho, sq_[1], sq_[2], sq_[3], sq_[4] + sq_[5] / (rho * P.rg)};
        for (int n = 0; n < 5; n++)
            if (b[n] != 0.0) atomicAdd(&pb[n * ch.pst], pscale * b[n]);
        return;
    }
    for (int n = 0; n < 6; n++)
        if (sq_[n] != 0.0) atomicAdd(&Qb[s + n * pl], sq_[n]);
}

__global__ void k_c2prim_vjp(const DevParams P, const double* __restrict__ U, const double* __restrict__ Qb,
                             double* out, double alpha, double beta) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    if (!(i >= NG && i < P.nx + NG && j >= NG && j < P.ny + NG && k >= NG && k < P.nz + NG)) return;
    const long long pl = P.plane;
    double u[5], qb[6], ub[5];
    for (int n = 0; n < 5; n++) u[n] = U[c + n * pl];
    for (int n = 0; n < 6; n++) qb[n] = Qb[c + n * pl];
    c2prim_vjp(P, u, qb, ub);
    for (int n = 0; n < 5; n++) {
        const double o = beta == 0.0 ? 0.0 : beta * out[c + n * pl];
        out[c + n * pl] = o + alpha * ub[n];
    }
}

// out = a x + b y over interior cells of U-layout arrays (RK3 adjoint combinations)
__global__ void k_axpby(const DevParams P, double* out, const double* x, double a, const double* y, double b) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    const bool in = i >= NG && i < P.nx + NG && j >= NG && j < P.ny + NG && k >= NG && k < P.nz + NG;
    for (int n = 0; n < 5; n++) {
        const long long o = c + n * P.plane;
        out[o] = in ? a * x[o] + (y ? b * y[o] : 0.0) : 0.0;
    }
}

// ---- launchers --------------------------------------------------------------------------
template <int DIR, bool CHAR> static cudaError_t launch_vjp_dir(const AdjArgs& a, cudaStream_t st) {
    constexpr int TL = VTile<DIR, CHAR>::TL, TC = VTile<DIR, CHAR>::TC;
    const DevParams& P = a.P;
    dim3 grid;
    if (DIR == 0) grid = dim3(cdiv(P.nx, TC), cdiv(P.ny, TL), P.nz);
    else if (DIR == 1) grid = dim3(cdiv(P.nx, TL), cdiv(P.ny, TC), P.nz);
    else grid = dim3(cdiv(P.nx, TL), cdiv(P.nz, TC), P.ny);
    k_sweep_vjp<DIR, CHAR><<<grid, VTile<DIR, CHAR>::NT, vjp_smem_bytes<DIR, CHAR>(), st>>>(a);
    return cudaGetLastError();
}

template <int DIR, bool CHAR> static cudaError_t configure_vjp() {
    return cudaFuncSetAttribute(k_sweep_vjp<DIR, CHAR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)vjp_smem_bytes<DIR, CHAR>());
}

cudaError_t adjoint_configure() {
    cudaError_t e;
    if ((e = configure_vjp<0, false>()) != cudaSuccess || (e = configure_vjp<1, false>()) != cudaSuccess ||
        (e = configure_vjp<2, false>()) != cudaSuccess || (e = configure_vjp<0, true>()) != cudaSuccess ||
        (e = configure_vjp<1, true>()) != cudaSuccess)
        return e;
    return configure_vjp<2, true>();
}

cudaError_t launch_sweep_vjp(int dir, const AdjArgs& a, cudaStream_t st) {
    const bool ch = a.P.character != 0;
    if (dir == 0) return ch ? launch_vjp_dir<0, true>(a, st) : launch_vjp_dir<0, false>(a, st);
    if (dir == 1) return ch ? launch_vjp_dir<1, true>(a, st) : launch_vjp_dir<1, false>(a, st);
    return ch ? launch_vjp_dir<2, true>(a, st) : launch_vjp_dir<2, false>(a, st);
}

static unsigned blocks_for(long long n, int t) { return (unsigned)((n + t - 1) / t); }

cudaError_t launch_viscous_vjp(const DevParams& P, const double* Q, const double* const m[9], const double* J,
                               const double* Lb, double* Fvb[3], double* gb, double* Qb, cudaStream_t st,
                               double* const mbar[9], double* Jbar, double mscale) {
    const long long nv = (long long)(P.nxt - 4) * (P.nyt - 4) * (P.nzt - 4);
    MetricBar mb;
    for (int n = 0; n < 9; n++) mb.m[n] = mbar ? mbar[n] : nullptr;
    mb.J = Jbar;
    mb.scale = mscale;
    k_visc_fvb<<<blocks_for(nv, 256), 256, 0, st>>>(P, Lb, J, Fvb[0], Fvb[1], Fvb[2]);
    k_visc_vjp<<<blocks_for(nv, 128), 128, 0, st>>>(P, Q, m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], J,
                                                     Fvb[0], Fvb[1], Fvb[2], gb, Qb, mb);
    k_visc_gather<<<blocks_for(P.plane, 256), 256, 0, st>>>(P, gb, Qb);
    return cudaGetLastError();
}

cudaError_t launch_jbar(const DevParams& P, const double* Lb, const double* L, const double* J, double* Jbar,
                        double mscale, cudaStream_t st) {
    k_jbar<<<blocks_for((long long)P.nx * P.ny * P.nz, 256), 256, 0, st>>>(P, Lb, L, J, Jbar, mscale);
    return cudaGetLastError();
}

cudaError_t launch_fill_vjp(const DevParams& P, const double* Q, double* Qb, double pscale, cudaStream_t st) {
    k_fill_vjp<<<blocks_for(P.plane, 256), 256, 0, st>>>(P, Q, Qb, pscale);
    return cudaGetLastError();
}

cudaError_t launch_c2prim_vjp(const DevParams& P, const double* U, const double* Qb, double* out, double alpha,
                              double beta, cudaStream_t st) {
    k_c2prim_vjp<<<blocks_for(P.plane, 256), 256, 0, st>>>(P, U, Qb, out, alpha, beta);
    return cudaGetLastError();
}

cudaError_t launch_axpby(const DevParams& P, double* out, const double* x, double a, const double* y, double b,
                         cudaStream_t st) {
    k_axpby<<<blocks_for(P.plane, 256), 256, 0, st>>>(P, out, x, a, y, b);
    return cudaGetLastError();
}

}  // namespace f3d
