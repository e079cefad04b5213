// k_sweep.cu — one direction of the inviscid RHS (plus that direction's viscous
// divergence) as a tiled sweep.
//
// A block owns TL grid lines along the sweep direction d and TC consecutive interior
// cells of each. Phase A splits the TC+8 cells the tile's stencils touch into Fp/Fm in
// shared memory (fluxSplit_*, split.jl), once per cell. Phase B reconstructs the TC+1
// faces of the tile, one thread per face, choosing UP7 / WENO7 / WENO5 / NND2 per face
// from the shock sensor (advect_x/xc and their y, z permutations, schemes.jl:86-1643).
// Phase C differences the face fluxes into the cells, adds the 4th-order central
// divergence of the viscous flux of direction d (div.jl:14-39), and accumulates into the
// RHS, or (last sweep) applies the Euler update and SSP-RK3 combination
// (div.jl:40-48, utils.jl:57-70) in place.
//
// Shared-memory layout is [var][line][pos] for d = x (threads run along the line) and
// [var][pos][line] for d = y, z (threads run across x-adjacent lines), so global loads
// coalesce along i and shared loads are conflict-free in both cases.
#include "f3d_face.cuh"
#include "f3d_sweep_epilogue.cuh"

namespace f3d {

// Tile (lines TL x cells TC), threads and resident blocks per SM of a sweep, by type.
// FP64: 8 x 64 in every direction on 288 threads, two blocks per SM (~76 KB of shared memory
// each): the tile's 8 x 72 split positions take exactly two rounds of 288 threads. Against
// 256 threads on 8 x 64 (xi) and 16 x 32 (eta, zeta) tiles, whose 576 / 640 positions took
// 2.25 / 2.5 rounds: +0.7% per RK3 step on the 256x64x64 shock tube (same box, three rounds
// of alternating builds); two blocks of nine warps leave 96 registers a thread (five warps on
// one of the SM's four register-file quarters), which the characteristic-wise instantiations
// use without spilling (72-92 component-wise). FP32:
// half-height tiles on 128 threads, six blocks per SM (~20 KB each): the same step time as
// three 256-thread blocks on that tube, 6% less per RHS on the component-wise tube and on
// the viscous vortex.
#ifndef SW_D_THREADS
#define SW_D_THREADS 288
#define SW_D_BLOCKS 2
#define SW_D_TL0 8
#define SW_D_TL12 8
#endif
#ifndef SW_D_TC0
#define SW_D_TC0 64
#define SW_D_TC12 64
#endif
template <int DIR, class R> struct Tile;
#ifndef SW_F_THREADS
#define SW_F_THREADS 128
#define SW_F_BLOCKS 6
#define SW_F_TL0 4
#define SW_F_TL12 8
#endif
template <> struct Tile<0, float> { static constexpr int TL = SW_F_TL0, TC = 64, NT = SW_F_THREADS, MINB = SW_F_BLOCKS; };
template <> struct Tile<1, float> { static constexpr int TL = SW_F_TL12, TC = 32, NT = SW_F_THREADS, MINB = SW_F_BLOCKS; };
template <> struct Tile<2, float> { static constexpr int TL = SW_F_TL12, TC = 32, NT = SW_F_THREADS, MINB = SW_F_BLOCKS; };
template <> struct Tile<0, double> { static constexpr int TL = SW_D_TL0, TC = SW_D_TC0, NT = SW_D_THREADS, MINB = SW_D_BLOCKS; };
template <> struct Tile<1, double> { static constexpr int TL = SW_D_TL12, TC = SW_D_TC12, NT = SW_D_THREADS, MINB = SW_D_BLOCKS; };
template <> struct Tile<2, double> { static constexpr int TL = SW_D_TL12, TC = SW_D_TC12, NT = SW_D_THREADS, MINB = SW_D_BLOCKS; };

template <int DIR, class R> constexpr size_t sweep_smem_bytes(bool hybrid) {
    using T = Tile<DIR, R>;
    return sizeof(R) * ((size_t)T::TL * (T::TC + 8) * (10 + (hybrid ? 1 : 0)) + (size_t)T::TL * (T::TC + 1) * 5) +
           sizeof(int) * (2 * (size_t)T::TL * (T::TC + 1) + 4);
}

template <int DIR, bool CHAR, class R>
__global__ void __launch_bounds__(Tile<DIR, R>::NT, Tile<DIR, R>::MINB) k_sweep(const SweepArgs a) {
    constexpr int TL = Tile<DIR, R>::TL, TC = Tile<DIR, R>::TC, NP = TC + 8, NF = TC + 1;
    constexpr int SWEEP_THREADS = Tile<DIR, R>::NT;
    const DevParams& P = a.P;
    const bool hybrid = P.fixed_branch < 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    R* sFp = reinterpret_cast<R*>(smem_raw);
    R* sFm = sFp + 5 * TL * NP;
    R* sF = sFm + 5 * TL * NP;
    R* sPhi = sF + 5 * TL * NF;
    const R* Qr = static_cast<const R*>(a.Q);
    const R* Ar[3] = {static_cast<const R*>(a.A[0]), static_cast<const R*>(a.A[1]), static_cast<const R*>(a.A[2])};
    const R* Hr[3] = {static_cast<const R*>(a.Ah[0]), static_cast<const R*>(a.Ah[1]),
                      static_cast<const R*>(a.Ah[2])};
    const R* Sr = static_cast<const R*>(a.S);
    const R* Phr = static_cast<const R*>(a.phi);

    // tile geometry: interior start c0 along d, first line l0 and line count
    const int Nd = DIR == 0 ? P.nx : (DIR == 1 ? P.ny : P.nz);
    const int Nl = DIR == 0 ? P.ny : P.nx;
    int c0, l0, other;
    if (DIR == 0) { c0 = blockIdx.x * TC; l0 = blockIdx.y * TL; other = blockIdx.z; }
    else { l0 = blockIdx.x * TL; c0 = blockIdx.y * TC; other = blockIdx.z; }
    const int nc = min(TC, Nd - c0);
    const int nl = min(TL, Nl - l0);
    const long long stride = DIR == 0 ? 1 : (DIR == 1 ? (long long)P.nxt : (long long)P.nxt * P.nyt);
    // linear index of (line l, full position along d = g)
    auto cell = [&](int l, int g) -> long long {
        if (DIR == 0) return lin3(P, g, l0 + l + NG, other + NG);
        if (DIR == 1) return lin3(P, l0 + l + NG, g, other + NG);
        return lin3(P, l0 + l + NG, other + NG, g);
    };
    auto sidx = [&](int l, int p) { return DIR == 0 ? l * NP + p : p * TL + l; };
    auto fidx = [&](int l, int t) { return DIR == 0 ? l * NF + t : t * TL + l; };
    const long long pl = P.plane;

    if (threadIdx.x < 2) reinterpret_cast<int*>(sPhi + TL * NP)[2 * TL * NF + threadIdx.x] = 0;
    // ---- Phase A: split every cell the tile's stencils reach (positions 0..nc+7, full
    // index c0 + p along d).
    for (int it = threadIdx.x; it < TL * NP; it += SWEEP_THREADS) {
        int l, p;
        if (DIR == 0) { l = it / NP; p = it - l * NP; } else { p = it / TL; l = it - p * TL; }
        if (l >= nl || p >= nc + 8) continue;
        const long long c = cell(l, c0 + p);
        R q[6];
#pragma unroll
        for (int n = 0; n < 6; n++) q[n] = Qr[c + n * pl];
        R fp[5], fm[5];
        split_cell<R>(P.split, cst<R>(P), q, split_sound<R>(P, a, c, q), Ar[0][c], Ar[1][c], Ar[2][c], Hr[0][c],
                      Hr[1][c], Hr[2][c], Sr[c], fp, fm);
        const int s = sidx(l, p);
#pragma unroll
        for (int n = 0; n < 5; n++) {
            sFp[n * TL * NP + s] = fp[n];
            sFm[n * TL * NP + s] = fm[n];
        }
        if (hybrid) sPhi[s] = Phr[c];
    }
    __syncthreads();

    // ---- Phase B: faces t = 0..nc (face t lies between positions t+3 and t+4).
    // With the hybrid switch, UP7 and NND2 faces are done at once and the WENO7 / WENO5
    // faces are queued and then processed by consecutive threads: near a shock only a few
    // faces of a warp take the long WENO paths, and done in place they would run with the
    // other lanes idle (and a warp holding both kinds would run both paths).
    auto do_face = [&](int l, int t, int br) {
        const long long cl = cell(l, c0 + t + 3), cr = cl + stride;
        R out[5];
        R s0 = R(0);
        if (br == 1 || br == 2) s0 = R(2) / (Sr[cl] + Sr[cr]);
        auto FP = [&](int n, int p) { return sFp[n * TL * NP + sidx(l, p)]; };
        auto FM = [&](int n, int p) { return sFm[n * TL * NP + sidx(l, p)]; };
        face_flux<CHAR, R>(P, a, br, t, s0, cl, cr, FP, FM, out);
        const int f = fidx(l, t);
#pragma unroll
        for (int n = 0; n < 5; n++) sF[n * TL * NF + f] = out[n];
        if (a.faces) {  // face-flux output in the reference's Fx/Fy/Fz shape
            const long long fx = P.nx + (DIR == 0), fy = P.ny + (DIR == 1), fz = P.nz + (DIR == 2);
            long long fi, fj, fk;
            if (DIR == 0) { fi = c0 + t; fj = l0 + l; fk = other; }
            else if (DIR == 1) { fi = l0 + l; fj = c0 + t; fk = other; }
            else { fi = l0 + l; fj = other; fk = c0 + t; }
            const long long fo = fi + fx * (fj + fy * fk), nf = fx * fy * fz;
#pragma unroll
            for (int n = 0; n < 5; n++) a.faces[fo + n * nf] = (double)out[n];
        }
    };
    int* list7 = reinterpret_cast<int*>(sPhi + TL * NP);
    int* list5 = list7 + TL * NF;
    int* counts = list5 + TL * NF;
    for (int it = threadIdx.x; it < TL * NF; it += SWEEP_THREADS) {
        int l, t;
        if (DIR == 0) { l = it / NF; t = it - l * NF; } else { t = it / TL; l = it - t * TL; }
        if (l >= nl || t > nc) continue;
        int br = P.fixed_branch;
        if (hybrid) {
            R ph[6];
#pragma unroll
            for (int o = 0; o < 6; o++) ph[o] = sPhi[sidx(l, t + 1 + o)];
            br = branch_of(P, ph);
            if (br == 1 || br == 2) {
                const int k = atomicAdd(&counts[br - 1], 1);
                (br == 1 ? list7 : list5)[k] = it;
                continue;
            }
        }
        do_face(l, t, br);
    }
    if (hybrid) {
        __syncthreads();
        const int n7 = counts[0], n5 = counts[1];
        for (int k = threadIdx.x; k < n7 + n5; k += SWEEP_THREADS) {
            const int it = k < n7 ? list7[k] : list5[k - n7];
            int l, t;
            if (DIR == 0) { l = it / NF; t = it - l * NF; } else { t = it / TL; l = it - t * TL; }
            do_face(l, t, k < n7 ? 1 : 2);
        }
    }
    if (a.out_mode == OUT_FACES) return;
    __syncthreads();

    // ---- Phase C: differences, viscous terms and the accumulation of out_mode.
    sweep_epilogue<DIR, TL, TC, SWEEP_THREADS, R>(a, sF, c0, l0, other, nc, nl, cell, fidx);
}

template <int DIR, bool CHAR, class R> static cudaError_t configure_dir() {
    return cudaFuncSetAttribute(k_sweep<DIR, CHAR, R>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sweep_smem_bytes<DIR, R>(true));
}

template <class R> static cudaError_t configure_type() {
    cudaError_t e;
    if ((e = configure_dir<0, false, R>()) != cudaSuccess) return e;
    if ((e = configure_dir<0, true, R>()) != cudaSuccess) return e;
    if ((e = configure_dir<1, false, R>()) != cudaSuccess) return e;
    if ((e = configure_dir<1, true, R>()) != cudaSuccess) return e;
    if ((e = configure_dir<2, false, R>()) != cudaSuccess) return e;
    return configure_dir<2, true, R>();
}

// Dynamic shared memory above 48 KB must be enabled per kernel before the first launch
// (and outside stream capture): called from f3d_create.
cudaError_t sweep_configure() {
    cudaError_t e = configure_type<double>();
    return e != cudaSuccess ? e : configure_type<float>();
}

template <int DIR, bool CHAR, class R> static cudaError_t launch_dir(const SweepArgs& a, cudaStream_t st) {
    constexpr int TL = Tile<DIR, R>::TL, TC = Tile<DIR, R>::TC;
    const DevParams& P = a.P;
    const size_t smem = sweep_smem_bytes<DIR, R>(true);
    dim3 grid;
    if (DIR == 0) grid = dim3(cdiv(P.nx, TC), cdiv(P.ny, TL), P.nz);
    else if (DIR == 1) grid = dim3(cdiv(P.nx, TL), cdiv(P.ny, TC), P.nz);
    else grid = dim3(cdiv(P.nx, TL), cdiv(P.nz, TC), P.ny);
    k_sweep<DIR, CHAR, R><<<grid, Tile<DIR, R>::NT, smem, st>>>(a);
    return cudaGetLastError();
}

template <class R> static cudaError_t launch_typed(int dir, const SweepArgs& a, cudaStream_t st) {
    const bool ch = a.P.character != 0;
    if (dir == 0) return ch ? launch_dir<0, true, R>(a, st) : launch_dir<0, false, R>(a, st);
    if (dir == 1) return ch ? launch_dir<1, true, R>(a, st) : launch_dir<1, false, R>(a, st);
    return ch ? launch_dir<2, true, R>(a, st) : launch_dir<2, false, R>(a, st);
}

cudaError_t launch_sweep(int dir, const SweepArgs& a, cudaStream_t st) {
    return a.fp32 ? launch_typed<float>(dir, a, st) : launch_typed<double>(dir, a, st);
}

}  // namespace f3d
