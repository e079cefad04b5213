// k_fvm.cu — the finite-volume RHS of FVM.jl (the reference's default, run.jl:64-65):
// face geometry from cell-centre coordinates, the hybrid switch on the shock sensor,
// linear / WENO7 / WENO5 / minmod reconstruction of the conserved variables U (component-
// wise, Conser_reconstruct_*, or in Roe-averaged characteristic fields, Eigen_reconstruct_*)
// and the HLLC flux (FVM.jl:1224-1357), differenced into the cells by the sweep epilogue
// shared with the finite-difference sweeps.
//
// k_face_geometry<d>: unit normal and area of every face of direction d, computed once per
//   grid (f3d_set_coordinates) and stored at the face's left cell. The operation order is
//   the oracle's and nothing is contracted into FMA, so the normals are bitwise those of
//   the restatement (the tangent basis of the characteristic fields switches on
//   |nz| <= |ny|, which must agree exactly).
// k_fvm_sweep<d, eigen>: tile of TL lines x TC cells. Phase A stages U and phi of the
//   TC+8 cells a line's faces reach; Phase B computes each face (linear faces at once, the
//   non-linear ones queued and then processed by consecutive threads); Phase C is the
//   shared epilogue (differences, viscous CD4, accumulation).
// k_stage_update: the RK update U = ca (U + dt J acc) + cb Un at interior cells. The
//   finite-volume sweeps read U, so the stage cannot update it inside the last sweep.
#include "f3d_kernels.cuh"
#include "f3d_sweep_epilogue.cuh"

namespace f3d {

// ------------------------------------------------------------------------------------
// geometry
template <int DIR>
__global__ void k_face_geometry(const DevParams P, const double* __restrict__ X, const double* __restrict__ Y,
                                const double* __restrict__ Z, double* gnx, double* gny, double* gnz, double* gar) {
    // faces f = 0..N_d of interior transverse lines; left cell full index f + NG - 1
    const int Nd = DIR == 0 ? P.nx : (DIR == 1 ? P.ny : P.nz);
    const int fa = DIR == 0 ? P.nx + 1 : P.nx, fb = DIR == 1 ? P.ny + 1 : P.ny;
    const long long nfaces = (long long)fa * fb * (DIR == 2 ? P.nz + 1 : P.nz);
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nfaces) return;
    (void)Nd;
    const int f0 = (int)(t % fa), f1 = (int)((t / fa) % fb), f2 = (int)(t / ((long long)fa * fb));
    int i = f0 + NG, j = f1 + NG, k = f2 + NG;
    if (DIR == 0) i -= 1;
    if (DIR == 1) j -= 1;
    if (DIR == 2) k -= 1;
    const long long sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const long long sd = DIR == 0 ? 1 : (DIR == 1 ? sy : sz);
    const long long sa = DIR == 0 ? sy : 1;             // transverse a: y for x faces, else x
    const long long sb = DIR == 2 ? sy : sz;            // transverse b: z, except y for z faces
    const long long c = lin3(P, i, j, k);
    // the cell at pa a + pb b from the face's left (side 0) or right (side 1) cell
    auto at = [&](const double* A, int pa, int pb, int side) { return A[c + side * sd + pa * sa + pb * sb]; };
    // 0.125 x the twelve centres summed left to right in the order of FVM.jl:16-21 (and the
    // j, k kernels): (pa,0), (0,pb), (pa,pb), each on both sides, then (-pa,0), (0,-pb),
    // (-pa,-pb) subtracted
    auto diag = [&](const double* A, int pa, int pb) {
        double s = __dadd_rn(at(A, pa, 0, 0), at(A, pa, 0, 1));
        s = __dadd_rn(s, at(A, 0, pb, 0));
        s = __dadd_rn(s, at(A, 0, pb, 1));
        s = __dadd_rn(s, at(A, pa, pb, 0));
        s = __dadd_rn(s, at(A, pa, pb, 1));
        s = __dsub_rn(s, at(A, -pa, 0, 0));
        s = __dsub_rn(s, at(A, -pa, 0, 1));
        s = __dsub_rn(s, at(A, 0, -pb, 0));
        s = __dsub_rn(s, at(A, 0, -pb, 1));
        s = __dsub_rn(s, at(A, -pa, -pb, 0));
        s = __dsub_rn(s, at(A, -pa, -pb, 1));
        return __dmul_rn(0.125, s);
    };
    const double dx1 = diag(X, 1, 1), dy1 = diag(Y, 1, 1), dz1 = diag(Z, 1, 1);
    const double dx2 = diag(X, -1, 1), dy2 = diag(Y, -1, 1), dz2 = diag(Z, -1, 1);
    const double sg = DIR == 1 ? -1.0 : 1.0;  // (a, b) = (x, z) on j faces: x cross z = -y
    double nx = __dmul_rn(__dmul_rn(sg, 0.5), __dadd_rn(__dmul_rn(dy1, dz2), -__dmul_rn(dz1, dy2)));
    double ny = __dmul_rn(__dmul_rn(sg, 0.5), __dadd_rn(__dmul_rn(dz1, dx2), -__dmul_rn(dx1, dz2)));
    double nz = __dmul_rn(__dmul_rn(sg, 0.5), __dadd_rn(__dmul_rn(dx1, dy2), -__dmul_rn(dy1, dx2)));
    const double area =
        __dsqrt_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(nx, nx), __dmul_rn(ny, ny)), __dmul_rn(nz, nz)), 1e-20));
    gnx[c] = __ddiv_rn(nx, area);
    gny[c] = __ddiv_rn(ny, area);
    gnz[c] = __ddiv_rn(nz, area);
    gar[c] = area;
}

cudaError_t launch_face_geometry(const DevParams& P, const double* x, const double* y, const double* z,
                                 double* const geo[12], cudaStream_t st) {
    const long long n0 = (long long)(P.nx + 1) * P.ny * P.nz, n1 = (long long)P.nx * (P.ny + 1) * P.nz,
                    n2 = (long long)P.nx * P.ny * (P.nz + 1);
    k_face_geometry<0><<<cdiv(n0, 128), 128, 0, st>>>(P, x, y, z, geo[0], geo[1], geo[2], geo[3]);
    k_face_geometry<1><<<cdiv(n1, 128), 128, 0, st>>>(P, x, y, z, geo[4], geo[5], geo[6], geo[7]);
    k_face_geometry<2><<<cdiv(n2, 128), 128, 0, st>>>(P, x, y, z, geo[8], geo[9], geo[10], geo[11]);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// face flux pieces (FVM.jl), double precision

// min / max that return NaN when either argument is NaN, as Julia's min and max do (the
// reference's wave-speed estimates): fmin/fmax would drop a NaN Roe speed and hide a
// negative reconstructed density from the non-finite check.
__device__ __forceinline__ double nan_min(double a, double b) { return a != a ? a : (b != b ? b : (b < a ? b : a)); }
__device__ __forceinline__ double nan_max(double a, double b) { return a != a ? a : (b != b ? b : (a < b ? b : a)); }

// HLLC flux along the unit normal n of the conserved states UL, UR (FVM.jl:1224-1357)
__device__ __forceinline__ void hllc(const DevParams& P, const double UL[5], const double UR[5], double nx,
                                     double ny, double nz, double F[5]) {
    const double g = P.gamma, gm = P.gm1;
    const double rL = UL[0], irL = 1.0 / rL;
    const double uL = UL[1] * irL, vL = UL[2] * irL, wL = UL[3] * irL, EL = UL[4];
    const double pL = gm * (EL - 0.5 * rL * (uL * uL + vL * vL + wL * wL));
    const double cL = sqrt(fabs(g * pL * irL));
    const double qL = uL * nx + vL * ny + wL * nz;
    const double rR = UR[0], irR = 1.0 / rR;
    const double uR = UR[1] * irR, vR = UR[2] * irR, wR = UR[3] * irR, ER = UR[4];
    const double pR = gm * (ER - 0.5 * rR * (uR * uR + vR * vR + wR * wR));
    const double cR = sqrt(fabs(g * pR * irR));
    const double qR = uR * nx + vR * ny + wR * nz;
    const double sL = sqrt(rL), sR = sqrt(rR), isum = 1.0 / (sL + sR);
    const double ur = (sL * uL + sR * uR) * isum, vr = (sL * vL + sR * vR) * isum, wr = (sL * wL + sR * wR) * isum;
    const double qr = ur * nx + vr * ny + wr * nz;
    const double HL = (EL + pL) * irL, HR = (ER + pR) * irR;
    const double Hr = (sL * HL + sR * HR) * isum;
    const double cr = sqrt(fabs(gm * (Hr - 0.5 * (ur * ur + vr * vr + wr * wr))));
    const double SL = nan_min(qL - cL, qr - cr);
    const double SR = nan_max(qR + cR, qr + cr);
    const double Ss = (pR - pL + rL * qL * (SL - qL) - rR * qR * (SR - qR)) / (rL * (SL - qL) - rR * (SR - qR) + 1e-12);
    const bool left = SL >= 0.0 || (SR > 0.0 && Ss >= 0.0);
    const double r = left ? rL : rR, u = left ? uL : uR, v = left ? vL : vR, w = left ? wL : wR;
    const double E = left ? EL : ER, p = left ? pL : pR, q = left ? qL : qR;
    F[0] = r * q;
    F[1] = r * u * q + p * nx;
    F[2] = r * v * q + p * ny;
    F[3] = r * w * q + p * nz;
    F[4] = (E + p) * q;
    if (SL >= 0.0 || SR <= 0.0) return;  // supersonic: the upwind state's physical flux
    // star state of the side: F* = F + S (U* - U)
    const double S = left ? SL : SR, ir = left ? irL : irR;
    const double* Us = left ? UL : UR;
    const double f = r * (S - q) / (S - Ss);
    const double st[5] = {f, f * (u + (Ss - q) * nx), f * (v + (Ss - q) * ny), f * (w + (Ss - q) * nz),
                          f * (E * ir + (Ss - q) * (Ss + p / (r * (S - q))))};
#pragma unroll
    for (int n = 0; n < 5; n++) F[n] += S * (st[n] - Us[n]);
}

// WENO7 / WENO5 / minmod of one side on a seven-point stencil in upwind order (FVM.jl)
__device__ __forceinline__ double fvm_weno7(const double V[7], double ss) {
    const double V1 = V[0], V2 = V[1], V3 = V[2], V4 = V[3], V5 = V[4], V6 = V[5], V7 = V[6];
    const double q1 = -3.0 * V1 + 13.0 * V2 - 23.0 * V3 + 25.0 * V4;
    const double q2 = V2 - 5.0 * V3 + 13.0 * V4 + 3.0 * V5;
    const double q3 = -V3 + 7.0 * V4 + 7.0 * V5 - V6;
    const double q4 = 3.0 * V4 + 13.0 * V5 - 5.0 * V6 + V7;
    double Is[4];  // the smoothness indicators in difference form (weno7_is, f3d_flux.cuh)
    weno7_is<double>(V, Is);
    const double I1 = Is[0], I2 = Is[1], I3 = Is[2], I4 = Is[3];
    // alpha_k = d_k / t_k^2 with t_k = 1e-10 + IS_k ss, normalised: one divide
    const double t1 = 1e-10 + I1 * ss, t2 = 1e-10 + I2 * ss, t3 = 1e-10 + I3 * ss, t4 = 1e-10 + I4 * ss;
    return weno7_combine(t1, t2, t3, t4, q1, q2, q3, q4) * (1.0 / 12.0);
}
__device__ __forceinline__ double fvm_weno5(const double V[7], double ss) {
    const double a = V[1], b = V[2], c = V[3], d = V[4], e = V[5];
    double t1 = a - 2.0 * b + c, t2 = a - 4.0 * b + 3.0 * c;
    const double s1 = 13.0 * t1 * t1 + 3.0 * t2 * t2;
    t1 = b - 2.0 * c + d;
    t2 = b - d;
    const double s2 = 13.0 * t1 * t1 + 3.0 * t2 * t2;
    t1 = c - 2.0 * d + e;
    t2 = 3.0 * c - 4.0 * d + e;
    const double s3 = 13.0 * t1 * t1 + 3.0 * t2 * t2;
    const double v1 = 2.0 * a - 7.0 * b + 11.0 * c, v2 = -b + 5.0 * c + 2.0 * d, v3 = 2.0 * c + 5.0 * d - e;
    return weno5_combine(1e-8 + s1 * ss, 1e-8 + s2 * ss, 1e-8 + s3 * ss, v1, v2, v3) * (1.0 / 6.0);
}
// br 1 = WENO7, 2 = WENO5, 3 = minmod; the two sides' minmod forms as FVM.jl:204-205
__device__ __forceinline__ double fvm_side(int br, bool right, const double V[7], double ss) {
    if (br == 1) return fvm_weno7(V, ss);
    if (br == 2) return fvm_weno5(V, ss);
    if (right) return V[3] - 0.5 * minmod(V[3] - V[2], V[3] - V[4]);
    return V[3] + 0.5 * minmod(V[3] - V[2], V[4] - V[3]);
}

// ------------------------------------------------------------------------------------
// the sweep
template <int DIR> struct FTile;
template <> struct FTile<0> { static constexpr int TL = 8, TC = 32; };
template <> struct FTile<1> { static constexpr int TL = 16, TC = 16; };
template <> struct FTile<2> { static constexpr int TL = 16, TC = 16; };
// Threads and resident blocks per SM of a sweep: the characteristic form holds ~250
// registers a thread, the component-wise one ~120. Small blocks let several blocks share an
// SM, so one block's barrier waits overlap another's face work.
#ifndef FVM_E_THREADS
#define FVM_E_THREADS 64
#define FVM_E_BLOCKS 4
#define FVM_C_THREADS 128
#define FVM_C_BLOCKS 2
#endif
template <bool EIGEN> struct FvmLaunch;
template <> struct FvmLaunch<true> { static constexpr int NT = FVM_E_THREADS, MINB = FVM_E_BLOCKS; };
template <> struct FvmLaunch<false> { static constexpr int NT = FVM_C_THREADS, MINB = FVM_C_BLOCKS; };

template <int DIR> constexpr size_t fvm_smem_bytes() {
    constexpr int TL = FTile<DIR>::TL, TC = FTile<DIR>::TC, NP = TC + 8, NF = TC + 1;
    return sizeof(double) * ((size_t)TL * NP * 6 + (size_t)TL * NF * 5) + sizeof(int) * ((size_t)TL * NF + 2);
}

template <int DIR, bool EIGEN>
__global__ void __launch_bounds__(FvmLaunch<EIGEN>::NT, FvmLaunch<EIGEN>::MINB) k_fvm_sweep(const SweepArgs a, const double* __restrict__ Ur,
                                                           const double* __restrict__ gnx, const double* __restrict__ gny,
                                                           const double* __restrict__ gnz, const double* __restrict__ gar) {
    constexpr int TL = FTile<DIR>::TL, TC = FTile<DIR>::TC, NP = TC + 8, NF = TC + 1;
    constexpr int FVM_THREADS = FvmLaunch<EIGEN>::NT;
    const DevParams& P = a.P;
    const bool hybrid = P.fixed_branch < 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double* sU = reinterpret_cast<double*>(smem_raw);  // [5][TL*NP]
    double* sPhi = sU + 5 * TL * NP;                    // [TL*NP]
    double* sF = sPhi + TL * NP;                        // [5][TL*NF]
    int* list = reinterpret_cast<int*>(sF + 5 * TL * NF);
    int* count = list + TL * NF;
    const double* Q = static_cast<const double*>(a.Q);
    const double* S = static_cast<const double*>(a.S);
    const double* Ph = static_cast<const double*>(a.phi);

    const int Nd = DIR == 0 ? P.nx : (DIR == 1 ? P.ny : P.nz);
    const int Nl = DIR == 0 ? P.ny : P.nx;
    int c0, l0, other;
    if (DIR == 0) { c0 = blockIdx.x * TC; l0 = blockIdx.y * TL; other = blockIdx.z; }
    else { l0 = blockIdx.x * TL; c0 = blockIdx.y * TC; other = blockIdx.z; }
    const int nc = min(TC, Nd - c0);
    const int nl = min(TL, Nl - l0);
    const long long stride = DIR == 0 ? 1 : (DIR == 1 ? (long long)P.nxt : (long long)P.nxt * P.nyt);
    auto cell = [&](int l, int g) -> long long {
        if (DIR == 0) return lin3(P, g, l0 + l + NG, other + NG);
        if (DIR == 1) return lin3(P, l0 + l + NG, g, other + NG);
        return lin3(P, l0 + l + NG, other + NG, g);
    };
    auto sidx = [&](int l, int p) { return DIR == 0 ? l * NP + p : p * TL + l; };
    auto fidx = [&](int l, int t) { return DIR == 0 ? l * NF + t : t * TL + l; };
    const long long pl = P.plane;

    if (threadIdx.x == 0) *count = 0;
    // Phase A: U and phi at positions 0..nc+7 (full index c0 + p along d)
    for (int it = threadIdx.x; it < TL * NP; it += FVM_THREADS) {
        int l, p;
        if (DIR == 0) { l = it / NP; p = it - l * NP; } else { p = it / TL; l = it - p * TL; }
        if (l >= nl || p >= nc + 8) continue;
        const long long c = cell(l, c0 + p);
        const int s = sidx(l, p);
#pragma unroll
        for (int n = 0; n < 5; n++) sU[n * TL * NP + s] = Ur[c + n * pl];
        if (hybrid) sPhi[s] = Ph[c];
    }
    __syncthreads();

    // Phase B: face t between positions t+3 (left cell, the kernels' i) and t+4
    auto face = [&](int l, int t, int br) {
        const long long cl = cell(l, c0 + t + 3);
        auto Uv = [&](int n, int p) { return sU[n * TL * NP + sidx(l, p)]; };
        const double nx = gnx[cl], ny = gny[cl], nz = gnz[cl];
        double UL[5], UR[5];
        if (br == 0) {  // linear scheme on U, FVM.jl:42-60
#pragma unroll
            for (int n = 0; n < 5; n++) {
                double vl = 0.0, vr = 0.0;
#pragma unroll
                for (int m = 0; m < 7; m++) {
                    vl += P.cd.lin[m] * Uv(n, t + m);
                    vr += P.cd.lin[m] * Uv(n, t + 7 - m);
                }
                UL[n] = vl;
                UR[n] = vr;
            }
        } else {
            const double ss = 2.0 / (S[cl + stride] + S[cl]);
            if (!EIGEN) {  // Conser_reconstruct, FVM.jl:739-855
#pragma unroll
                for (int n = 0; n < 5; n++) {
                    double VL[7], VR[7];
#pragma unroll
                    for (int m = 0; m < 7; m++) {
                        VL[m] = Uv(n, t + m);
                        VR[m] = Uv(n, t + 7 - m);
                    }
                    UL[n] = fvm_side(br, false, VL, ss);
                    UR[n] = fvm_side(br, true, VR, ss);
                }
            } else {  // Eigen_reconstruct, FVM.jl:65-228
                const double rl = Q[cl], rr = Q[cl + stride];
                const double srl = sqrt(rl), srr = sqrt(rr), isr = 1.0 / (srl + srr);
                const double u = (srl * Q[cl + pl] + srr * Q[cl + stride + pl]) * isr;
                const double v = (srl * Q[cl + 2 * pl] + srr * Q[cl + stride + 2 * pl]) * isr;
                const double w = (srl * Q[cl + 3 * pl] + srr * Q[cl + stride + 3 * pl]) * isr;
                const double gg = P.gamma / P.gm1;
                auto Hof = [&](long long c) {
                    const double uu = Q[c + pl], vv = Q[c + 2 * pl], ww = Q[c + 3 * pl];
                    return gg * Q[c + 4 * pl] / Q[c] + 0.5 * (uu * uu + vv * vv + ww * ww);
                };
                const double H = (srl * Hof(cl) + srr * Hof(cl + stride)) * isr;
                const double v2 = 0.5 * (u * u + v * v + w * w);
                const double c = sqrt(P.gm1 * (H - v2));
                double lx, ly, lz;
                if (fabs(nz) <= fabs(ny)) {
                    const double id = 1.0 / sqrt(nx * nx + ny * ny + 1e-12);
                    lx = -ny * id; ly = nx * id; lz = 0.0;
                } else {
                    const double id = 1.0 / sqrt(nx * nx + nz * nz + 1e-12);
                    lx = -nz * id; ly = 0.0; lz = nx * id;
                }
                const double mx = ny * lz - nz * ly, my = nz * lx - nx * lz, mz = nx * ly - ny * lx;
                const double invc = 1.0 / c, invc2 = invc * invc, K = P.gm1;
                const double Ku = K * u * invc2, Kv = K * v * invc2, Kw = K * w * invc2;
                const double Kv2 = K * v2 * invc2, Kc2 = K * invc2;
                const double un = u * nx + v * ny + w * nz, ul = u * lx + v * ly + w * lz,
                             um = u * mx + v * my + w * mz;
                const double uni = un * invc, nxi = nx * invc, nyi = ny * invc, nzi = nz * invc;
#pragma unroll
                for (int q = 0; q < 5; q++) { UL[q] = 0.0; UR[q] = 0.0; }
#pragma unroll 1
                for (int n = 0; n < 5; n++) {
                    double ln[5], rn[5];
                    if (n == 0) {
                        ln[0] = 0.5 * (Kv2 + uni); ln[1] = -0.5 * (Ku + nxi); ln[2] = -0.5 * (Kv + nyi);
                        ln[3] = -0.5 * (Kw + nzi); ln[4] = 0.5 * Kc2;
                        rn[0] = 1.0; rn[1] = u - nx * c; rn[2] = v - ny * c; rn[3] = w - nz * c; rn[4] = H - un * c;
                    } else if (n == 1) {
                        ln[0] = 1.0 - Kv2; ln[1] = Ku; ln[2] = Kv; ln[3] = Kw; ln[4] = -Kc2;
                        rn[0] = 1.0; rn[1] = u; rn[2] = v; rn[3] = w; rn[4] = v2;
                    } else if (n == 2) {
                        ln[0] = 0.5 * (Kv2 - uni); ln[1] = -0.5 * (Ku - nxi); ln[2] = -0.5 * (Kv - nyi);
                        ln[3] = -0.5 * (Kw - nzi); ln[4] = 0.5 * Kc2;
                        rn[0] = 1.0; rn[1] = u + nx * c; rn[2] = v + ny * c; rn[3] = w + nz * c; rn[4] = H + un * c;
                    } else if (n == 3) {
                        ln[0] = -ul; ln[1] = lx; ln[2] = ly; ln[3] = lz; ln[4] = 0.0;
                        rn[0] = 0.0; rn[1] = lx; rn[2] = ly; rn[3] = lz; rn[4] = ul;
                    } else {
                        ln[0] = -um; ln[1] = mx; ln[2] = my; ln[3] = mz; ln[4] = 0.0;
                        rn[0] = 0.0; rn[1] = mx; rn[2] = my; rn[3] = mz; rn[4] = um;
                    }
                    double VL[7], VR[7];
#pragma unroll
                    for (int m = 0; m < 7; m++) {
                        double sl = 0.0, sr = 0.0;
#pragma unroll
                        for (int q = 0; q < 5; q++) {
                            sl += ln[q] * Uv(q, t + m);
                            sr += ln[q] * Uv(q, t + 7 - m);
                        }
                        VL[m] = sl;
                        VR[m] = sr;
                    }
                    const double vl = fvm_side(br, false, VL, ss), vr = fvm_side(br, true, VR, ss);
#pragma unroll
                    for (int q = 0; q < 5; q++) {
                        UL[q] += rn[q] * vl;
                        UR[q] += rn[q] * vr;
                    }
                }
            }
        }
        double Ff[5];
        hllc(P, UL, UR, nx, ny, nz, Ff);
        const double ar = gar[cl];
        const int f = fidx(l, t);
#pragma unroll
        for (int n = 0; n < 5; n++) sF[n * TL * NF + f] = Ff[n] * ar;
        if (a.faces) {  // face-flux output in the reference's Fx/Fy/Fz shape
            const long long fx = P.nx + (DIR == 0), fy = P.ny + (DIR == 1), fz = P.nz + (DIR == 2);
            long long fi, fj, fk;
            if (DIR == 0) { fi = c0 + t; fj = l0 + l; fk = other; }
            else if (DIR == 1) { fi = l0 + l; fj = c0 + t; fk = other; }
            else { fi = l0 + l; fj = other; fk = c0 + t; }
            const long long fo = fi + fx * (fj + fy * fk), nf = fx * fy * fz;
#pragma unroll
            for (int n = 0; n < 5; n++) a.faces[fo + n * nf] = Ff[n] * ar;
        }
    };
    for (int it = threadIdx.x; it < TL * NF; it += FVM_THREADS) {
        int l, t;
        if (DIR == 0) { l = it / NF; t = it - l * NF; } else { t = it / TL; l = it - t * TL; }
        if (l >= nl || t > nc) continue;
        int br = P.fixed_branch;
        if (hybrid) {  // max of phi over cells i-2..i+3 (FVM.jl:33)
            double ph[6];
#pragma unroll
            for (int o = 0; o < 6; o++) ph[o] = sPhi[sidx(l, t + 1 + o)];
            br = branch_of(P, ph);
        }
        if (br != 0) {
            list[atomicAdd(count, 1)] = it * 4 + br;
            continue;
        }
        face(l, t, 0);
    }
    __syncthreads();
    const int nq = *count;
    for (int k = threadIdx.x; k < nq; k += FVM_THREADS) {
        const int e = list[k], it = e >> 2;
        int l, t;
        if (DIR == 0) { l = it / NF; t = it - l * NF; } else { t = it / TL; l = it - t * TL; }
        face(l, t, e & 3);
    }
    if (a.out_mode == OUT_FACES) return;
    __syncthreads();
    // Phase C
    sweep_epilogue<DIR, TL, TC, FVM_THREADS, double>(a, sF, c0, l0, other, nc, nl, cell, fidx);
}

template <int DIR, bool EIGEN> static cudaError_t fvm_configure_one() {
    return cudaFuncSetAttribute(k_fvm_sweep<DIR, EIGEN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)fvm_smem_bytes<DIR>());
}

cudaError_t fvm_configure() {
    cudaError_t e;
    if ((e = fvm_configure_one<0, true>()) != cudaSuccess) return e;
    if ((e = fvm_configure_one<0, false>()) != cudaSuccess) return e;
    if ((e = fvm_configure_one<1, true>()) != cudaSuccess) return e;
    if ((e = fvm_configure_one<1, false>()) != cudaSuccess) return e;
    if ((e = fvm_configure_one<2, true>()) != cudaSuccess) return e;
    return fvm_configure_one<2, false>();
}

template <int DIR, bool EIGEN>
static cudaError_t fvm_launch_dir(const SweepArgs& a, const double* U, const double* const geo[12], cudaStream_t st) {
    constexpr int TL = FTile<DIR>::TL, TC = FTile<DIR>::TC;
    const DevParams& P = a.P;
    dim3 grid;
    if (DIR == 0) grid = dim3(cdiv(P.nx, TC), cdiv(P.ny, TL), P.nz);
    else if (DIR == 1) grid = dim3(cdiv(P.nx, TL), cdiv(P.ny, TC), P.nz);
    else grid = dim3(cdiv(P.nx, TL), cdiv(P.nz, TC), P.ny);
    const double* const* g = geo + 4 * DIR;
    k_fvm_sweep<DIR, EIGEN><<<grid, FvmLaunch<EIGEN>::NT, fvm_smem_bytes<DIR>(), st>>>(a, U, g[0], g[1], g[2], g[3]);
    return cudaGetLastError();
}

cudaError_t launch_fvm_sweep(int dir, bool eigen, const SweepArgs& a, const double* U, const double* const geo[12],
                             cudaStream_t st) {
    if (dir == 0) return eigen ? fvm_launch_dir<0, true>(a, U, geo, st) : fvm_launch_dir<0, false>(a, U, geo, st);
    if (dir == 1) return eigen ? fvm_launch_dir<1, true>(a, U, geo, st) : fvm_launch_dir<1, false>(a, U, geo, st);
    return eigen ? fvm_launch_dir<2, true>(a, U, geo, st) : fvm_launch_dir<2, false>(a, U, geo, st);
}

// ------------------------------------------------------------------------------------
// RK update from the accumulated RHS (div.jl:1-50 fused with linComb, utils.jl:57-70)
__global__ void k_stage_update(const DevParams P, const double* __restrict__ acc, const double* __restrict__ J,
                               double dt, double* U, double* Un, int stage1_copy, int combine, double ca, double cb,
                               const double* __restrict__ dtl) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)P.nx * P.ny * P.nz;
    if (t >= n) return;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    const long long c = lin3(P, i + NG, j + NG, k + NG), pl = P.plane;
    const double Jact = J[c] * (dtl ? dtl[c] : dt);
#pragma unroll
    for (int v = 0; v < 5; v++) {
        const double u = U[c + v * pl];
        if (stage1_copy) Un[c + v * pl] = u;
        double un = u + acc[c + v * pl] * Jact;
        if (combine) un = un * ca + Un[c + v * pl] * cb;
        U[c + v * pl] = un;
    }
}

cudaError_t launch_stage_update(const DevParams& P, const double* acc, const double* J, double dt, double* U,
                                double* Un, int stage1_copy, int combine, double ca, double cb, cudaStream_t st,
                                const double* dtl) {
    const long long n = (long long)P.nx * P.ny * P.nz;
    k_stage_update<<<cdiv(n, 256), 256, 0, st>>>(P, acc, J, dt, U, Un, stage1_copy, combine, ca, cb, dtl);
    return cudaGetLastError();
}

}  // namespace f3d
