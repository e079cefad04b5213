// k_sweep_tma.cu — the mixed-precision (FP32) finite-difference sweeps with their stencil
// tiles staged by the Tensor Memory Accelerator.
//
// Same numerics and phases as k_sweep.cu (split in Phase A, face reconstruction in Phase B,
// differences and accumulation in Phase C), but:
//  - the inputs of Phase A (the FP32 primitive state, the metric row of the sweep direction
//    with A/|A| and |A|, and the sensor) arrive as three tensor tiles, box = the tile's TL
//    lines x (TC + 8) positions with their 4-cell halos, copied by cp.async.bulk.tensor into
//    shared memory and completed on an mbarrier; the boxes land in the [var][line][pos] /
//    [var][pos][line] layouts the phases index, so no thread issues a global load for them;
//  - in the last sweep of an RHS (the zeta sweep), the inputs of Phase C (the two FP32
//    direction sums, J and, for a stage, U and Un) arrive the same way on a second mbarrier,
//    issued as soon as the previous tile's Phase C is done;
//  - blocks are persistent: each takes its next tile from a counter of the launch (atomicAdd;
//    the shock-capturing faces cluster in a few tile columns, so a static assignment would
//    leave some blocks with all of them) and issues that tile's copies as soon as Phase A has
//    consumed the current one, so the loads overlap Phases B and C.
// Every mbarrier wait is bounded (time and iterations); a wait that gives up sets bit 0 of
// the context's kernel-status word, waits (bounded) for the copy in flight and ends the
// block, and the host reports F3D_ERR_CUDA at its next status check.
//
// Used for F3D_PREC_MIXED when the x extent with ghosts is a multiple of 4 (16-byte rows of
// FP32, as the tensor copies need); other grids take the direct-load sweeps.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "f3d_face.cuh"
#include "f3d_sweep_epilogue.cuh"

namespace f3d {

// Tiles of the TMA sweeps: xi 4 lines x 64 cells, eta / zeta 8 x-adjacent lines x 32 cells,
// 128 threads (as the direct-load FP32 sweeps). The x extent of an eta / zeta box (TL floats)
// must be a multiple of 4 and its x origin (first line + 4) too: TL a multiple of 4.
#ifndef TMA_NT
#define TMA_NT 128
#define TMA_MINB 5
#define TMA_TL0 4
#define TMA_TC0 64
#define TMA_TL12 8
#define TMA_TC12 32
#endif
template <int DIR> struct TTile;
template <> struct TTile<0> { static constexpr int TL = TMA_TL0, TC = TMA_TC0, NT = TMA_NT, MINB = TMA_MINB; };
template <> struct TTile<1> { static constexpr int TL = TMA_TL12, TC = TMA_TC12, NT = TMA_NT, MINB = TMA_MINB; };
template <> struct TTile<2> { static constexpr int TL = TMA_TL12, TC = TMA_TC12, NT = TMA_NT, MINB = TMA_MINB; };
static_assert(TMA_TL12 % 4 == 0 && TMA_TC0 % 4 == 0, "TMA boxes need 16-byte x extents and origins");

constexpr int kQVars = 6;     // rho, u, v, w, p, T
constexpr int kMetVars = 7;   // A1, A2, A3, A1/|A|, A2/|A|, A3/|A|, |A| of the sweep direction

template <int DIR, bool EPI = false> struct TmaLayout {
    static constexpr int TL = TTile<DIR>::TL, TC = TTile<DIR>::TC, NP = TC + 8, NF = TC + 1;
    static constexpr int BOX = TL * NP;                                   // floats per variable
    static constexpr size_t raw_q = 0;                                    // 6 x BOX
    static constexpr size_t raw_m = raw_q + sizeof(float) * kQVars * BOX; // 7 x BOX
    static constexpr size_t raw_phi = raw_m + sizeof(float) * kMetVars * BOX;
    static constexpr size_t raw_end = raw_phi + sizeof(float) * BOX;
    static constexpr size_t fp = (raw_end + 127) & ~(size_t)127;          // split fluxes 10 x BOX
    static constexpr size_t ff = fp + sizeof(float) * 10 * BOX;           // face fluxes 5 x TL x NF
    static constexpr size_t phi = ff + sizeof(float) * 5 * TL * NF;       // sensor, BOX
    static constexpr size_t sabs = phi + sizeof(float) * BOX;             // |A|, BOX
    static constexpr size_t lists = sabs + sizeof(float) * BOX;           // 2 x TL x NF ints + 4
    static constexpr size_t bar = (lists + sizeof(int) * (2 * TL * NF + 6) + 7) & ~(size_t)7;
    // staged Phase C inputs of the last sweep (EPI): boxes of the tile's TL x TC interior cells
    static constexpr int CELLS = TL * TC;
    static constexpr size_t e_acc = (bar + 16 + 127) & ~(size_t)127;       // 5 x CELLS floats
    static constexpr size_t e_acc2 = e_acc + sizeof(float) * 5 * CELLS;    // 5 x CELLS floats
    static constexpr size_t e_J = e_acc2 + sizeof(float) * 5 * CELLS;      // CELLS doubles
    static constexpr size_t e_U = e_J + sizeof(double) * CELLS;            // 5 x CELLS doubles
    static constexpr size_t e_Un = e_U + sizeof(double) * 5 * CELLS;       // 5 x CELLS doubles
    static constexpr size_t total = EPI ? e_Un + sizeof(double) * 5 * CELLS : bar + 16;
    static constexpr unsigned epi_rhs_bytes = (unsigned)(sizeof(float) * 10 * CELLS + sizeof(double) * CELLS);
    static constexpr unsigned epi_u_bytes = (unsigned)(sizeof(double) * 5 * CELLS);
    static_assert((sizeof(float) * CELLS) % 128 == 0, "staged Phase C boxes must start 128-byte aligned");
    // bytes one tile's copies deliver (complete_tx counts whole boxes, filled or not)
    static constexpr unsigned tx_bytes = (unsigned)(sizeof(float) * (kQVars + kMetVars + 1) * BOX);
    static_assert((sizeof(float) * BOX) % 128 == 0, "every box must start 128-byte aligned");
};

// ---- TMA and mbarrier primitives (inline PTX) -------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// order this thread's (generic-proxy) shared-memory accesses before later async-proxy copies
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait for the phase `parity` of bar: gives up after limit_ns of wall time or 2^26
// polls, whichever comes first. Returns true when the phase completed.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
    const unsigned long long t0 = globaltimer_ns();
    for (unsigned it = 0; it < (1u << 26); it++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((it & 255u) == 255u && globaltimer_ns() - t0 > limit_ns) return false;
    }
    return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, unsigned long long* bar, int x, int y,
                                            int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z),
        "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, unsigned long long* bar, int x, int y,
                                            int z, int w) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
        : "memory");
}

// Tensor maps of one direction: Q32 (x, y, z, 6), the direction's metric pack (x, y, z, 7)
// and the sensor (x, y, z). Boxes: xi (NP, TL, 1[, n]), eta (TL, NP, 1[, n]), zeta (TL, 1, NP[, n]).
struct SweepMaps {  // CUtensorMap is 64-byte aligned
    CUtensorMap q, m, phi;
};
// Phase C inputs of the last sweep: the FP32 direction sums (x, y, z, 5) x 2, J (x, y, z) and
// U, Un (x, y, z, 5) in FP64; box (TL, 1, TC[, n]) of the zeta tile's interior cells
struct EpiMaps {
    CUtensorMap acc, acc2, J, U, Un;
};

constexpr unsigned long long kWaitLimitNs = 2000000000ull;  // 2 s: a tile copy takes microseconds

template <int DIR, bool CHAR, bool EPI>
__global__ void __launch_bounds__(TTile<DIR>::NT, TTile<DIR>::MINB)
    k_sweep_tma(const __grid_constant__ SweepArgs a, const __grid_constant__ SweepMaps maps,
                const __grid_constant__ EpiMaps em) {
    static_assert(!EPI || DIR == 2, "Phase C is staged in the last (zeta) sweep only");
    using L = TmaLayout<DIR, EPI>;
    constexpr int TL = L::TL, TC = L::TC, NP = L::NP, NF = L::NF, BOX = L::BOX, NT = TTile<DIR>::NT;
    const DevParams& P = a.P;
    const bool hybrid = P.fixed_branch < 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    float* rq = reinterpret_cast<float*>(smem_raw + L::raw_q);
    float* rm = reinterpret_cast<float*>(smem_raw + L::raw_m);
    float* rphi = reinterpret_cast<float*>(smem_raw + L::raw_phi);
    float* sFp = reinterpret_cast<float*>(smem_raw + L::fp);
    float* sFm = sFp + 5 * BOX;
    float* sF = reinterpret_cast<float*>(smem_raw + L::ff);
    float* sPhi = reinterpret_cast<float*>(smem_raw + L::phi);
    float* sS = reinterpret_cast<float*>(smem_raw + L::sabs);
    int* list7 = reinterpret_cast<int*>(smem_raw + L::lists);
    int* list5 = list7 + TL * NF;
    int* counts = list5 + TL * NF;  // counts[0..1]: WENO7 / WENO5 queue lengths; counts[4]: next tile
    unsigned long long* bar = reinterpret_cast<unsigned long long*>(smem_raw + L::bar);
    unsigned long long* ebar = bar + 1;  // the staged Phase C inputs (EPI)
    const bool stage = a.out_mode == OUT_STAGE;

    const int Nd = DIR == 0 ? P.nx : (DIR == 1 ? P.ny : P.nz);
    const int Nl = DIR == 0 ? P.ny : P.nx;
    const int No = DIR == 2 ? P.ny : P.nz;  // the third (outer) direction of the tile grid
    const int tiles_c = (Nd + TC - 1) / TC, tiles_l = (Nl + TL - 1) / TL;
    const int ntiles = tiles_c * tiles_l * No;
    const long long stride = DIR == 0 ? 1 : (DIR == 1 ? (long long)P.nxt : (long long)P.nxt * P.nyt);
    auto sidx = [&](int l, int p) { return DIR == 0 ? l * NP + p : p * TL + l; };
    auto fidx = [&](int l, int t) { return DIR == 0 ? l * NF + t : t * TL + l; };
    // tile id -> (c0, l0, other): cell blocks fastest, then line blocks, then the outer index
    auto decode = [&](int tid, int& c0, int& l0, int& other) {
        const int cb = tid % tiles_c, r = tid / tiles_c;
        c0 = cb * TC;
        l0 = (r % tiles_l) * TL;
        other = r / tiles_l;
    };
    auto issue = [&](int tid) {  // one thread: the three tensor copies of tile tid
        int c0, l0, other;
        decode(tid, c0, l0, other);
        int x, y, z;
        if (DIR == 0) { x = c0; y = l0 + NG; z = other + NG; }
        else if (DIR == 1) { x = l0 + NG; y = c0; z = other + NG; }
        else { x = l0 + NG; y = other + NG; z = c0; }
        fence_proxy_async();
        mbar_expect_tx(bar, L::tx_bytes);
        tma_load_4d(rq, &maps.q, bar, x, y, z, 0);
        tma_load_4d(rm, &maps.m, bar, x, y, z, 0);
        tma_load_3d(rphi, &maps.phi, bar, x, y, z);
    };

    auto issue_epi = [&](int tid) {  // one thread: the Phase C copies of tile tid (EPI)
        int c0, l0, other;
        decode(tid, c0, l0, other);
        const int x = l0 + NG, y = other + NG, z = c0 + NG;
        fence_proxy_async();
        mbar_expect_tx(ebar, L::epi_rhs_bytes + (stage ? L::epi_u_bytes * (a.combine ? 2u : 1u) : 0u));
        tma_load_4d(smem_raw + L::e_acc, &em.acc, ebar, x, y, z, 0);
        tma_load_4d(smem_raw + L::e_acc2, &em.acc2, ebar, x, y, z, 0);
        tma_load_3d(smem_raw + L::e_J, &em.J, ebar, x, y, z);
        if (stage) {
            tma_load_4d(smem_raw + L::e_U, &em.U, ebar, x, y, z, 0);
            if (a.combine) tma_load_4d(smem_raw + L::e_Un, &em.Un, ebar, x, y, z, 0);
        }
    };
    // L2 prefetch of the rows Phase C reads for tile tid (the accumulators, J and, for a
    // stage, U and Un): one prefetch per row of the tile's first and last line (rows of TL
    // x-adjacent cells for eta / zeta; for xi, every 16 cells of a line)
    auto prefetch_epilogue = [&](int tid) {
        if (tid >= ntiles) return;
        int c0, l0, other;
        decode(tid, c0, l0, other);
        const bool stage = a.out_mode == OUT_STAGE;
        const int narr = 11 + (stage ? 10 : 0);  // acc 5, acc2 5, J 1, U 5, Un 5
        const int nrow = DIR == 0 ? TL * (TC / 16) : 2 * TC;
        for (int it = threadIdx.x; it < nrow * narr; it += NT) {
            const int row = it % nrow, k = it / nrow;
            int l, t;
            if (DIR == 0) { l = row / (TC / 16); t = (row % (TC / 16)) * 16; }
            else { t = row >> 1; l = (row & 1) ? TL - 1 : 0; }
            long long c;
            if (DIR == 0) c = lin3(P, c0 + t + NG, l0 + l + NG, other + NG);
            else if (DIR == 1) c = lin3(P, l0 + l + NG, c0 + t + NG, other + NG);
            else c = lin3(P, l0 + l + NG, other + NG, c0 + t + NG);
            if (c >= P.plane) continue;  // lines beyond the grid on a ragged last tile
            const void* addr;
            if (k < 5) addr = static_cast<const float*>(a.acc) + c + k * P.plane;
            else if (k < 10) addr = a.acc2 ? a.acc2 + c + (k - 5) * P.plane : nullptr;
            else if (k == 10) addr = a.J + c;
            else if (k < 16) addr = a.U + c + (k - 11) * P.plane;
            else addr = a.combine ? a.Un + c + (k - 16) * P.plane : nullptr;
            if (addr) asm volatile("prefetch.global.L2 [%0];" ::"l"(addr));
        }
    };
    // Phase C of the last sweep from the staged boxes ([n][t][l]: cell (l, t) of the tile):
    // the face-flux difference and the CD4 viscous divergence (Fv from global memory), the
    // compensated sum of the three directions, then J x L (OUT_RHS) or the RK update in FP64
    auto staged_epilogue = [&](int c0, int l0, int other, int nc, int nl) {
        const float* eacc = reinterpret_cast<const float*>(smem_raw + L::e_acc);
        const float* eacc2 = reinterpret_cast<const float*>(smem_raw + L::e_acc2);
        const double* eJ = reinterpret_cast<const double*>(smem_raw + L::e_J);
        const double* eU = reinterpret_cast<const double*>(smem_raw + L::e_U);
        const double* eUn = reinterpret_cast<const double*>(smem_raw + L::e_Un);
        constexpr int CELLS = L::CELLS;
        const long long pl = P.plane;
        const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
        const long long vplane = (long long)vxt * vyt * vzt;
        const float* Fvr = static_cast<const float*>(a.Fv);
        for (int it = threadIdx.x; it < CELLS; it += NT) {
            const int t = it / TL, l = it - t * TL;
            if (l >= nl || t >= nc) continue;
            const long long c = lin3(P, l0 + l + NG, other + NG, c0 + t + NG);
            float d[5];
#pragma unroll
            for (int n = 0; n < 5; n++) d[n] = sF[n * TL * NF + fidx(l, t)] - sF[n * TL * NF + fidx(l, t + 1)];
            if (Fvr) {  // Fv index = full index - 2 in every dimension (viscous.jl:119, div.jl:14-39)
                const long long vc = (l0 + l + NG - 2) + (long long)vxt * ((other + NG - 2) + (long long)vyt * (c0 + t + NG - 2));
                const long long vs = (long long)vxt * vyt;
                const float k1 = 1.f / 12.f, k2 = -2.f / 3.f;
#pragma unroll
                for (int n = 0; n < 4; n++) {
                    const float* F = Fvr + n * vplane + vc;
                    d[n + 1] += k1 * (F[-2 * vs] - F[2 * vs]) + k2 * (F[-vs] - F[vs]);
                }
            }
            double L5[5];
#pragma unroll
            for (int n = 0; n < 5; n++)
                L5[n] = to_f64(sum3_compensated(eacc[n * CELLS + it], eacc2[n * CELLS + it], d[n]));
            if (!stage) {
                const double Jc = eJ[it];
#pragma unroll
                for (int n = 0; n < 5; n++) a.out[c + n * pl] = Jc * L5[n];
            } else {
                const double Jact = eJ[it] * a.dt;
#pragma unroll
                for (int n = 0; n < 5; n++) {
                    const double u = eU[n * CELLS + it];
                    if (a.stage1_copy) a.Un[c + n * pl] = u;
                    double un = u + L5[n] * Jact;
                    if (a.combine) un = un * a.ca + eUn[n * CELLS + it] * a.cb;
                    a.U[c + n * pl] = un;
                }
            }
        }
    };
    unsigned* ctr = a.tile_ctr + DIR;  // zeroed before the three sweeps of an RHS
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        if (EPI) mbar_init(ebar, 1);
        fence_mbar_init();
        const int first = (int)atomicAdd(ctr, 1u);
        counts[4] = first;
        if (first < ntiles) {
            issue(first);
            if (EPI) issue_epi(first);
        }
    }
    __syncthreads();
    int tile = counts[4];
    unsigned parity = 0;
    for (; tile < ntiles; parity ^= 1u) {
        int c0, l0, other;
        decode(tile, c0, l0, other);
        const int nc = min(TC, Nd - c0), nl = min(TL, Nl - l0);
        auto cell = [&](int l, int g) -> long long {
            if (DIR == 0) return lin3(P, g, l0 + l + NG, other + NG);
            if (DIR == 1) return lin3(P, l0 + l + NG, g, other + NG);
            return lin3(P, l0 + l + NG, other + NG, g);
        };
        // wait for this tile's copies (thread 0, bounded), then release the block
        int timed_out = 0;
        if (threadIdx.x == 0) {
            timed_out = !mbar_wait_bounded(bar, parity, kWaitLimitNs);
            if (timed_out) {  // drain what may be in flight (this tile's copies), bounded again
                atomicOr(a.kstat, 1u);
                mbar_wait_bounded(bar, parity, kWaitLimitNs);
                if (EPI) mbar_wait_bounded(ebar, parity, kWaitLimitNs);
            }
            counts[0] = 0;
            counts[1] = 0;
        }
        if (__syncthreads_or(timed_out)) return;

        // ---- Phase A: split every staged position (0..nc+7) into Fp/Fm
        for (int it = threadIdx.x; it < BOX; it += NT) {
            int l, p;
            if (DIR == 0) { l = it / NP; p = it - l * NP; } else { p = it / TL; l = it - p * TL; }
            if (l >= nl || p >= nc + 8) continue;
            const int s = sidx(l, p);
            float q[6];
#pragma unroll
            for (int n = 0; n < 6; n++) q[n] = rq[n * BOX + s];
            float fp[5], fm[5];
            split_cell<float>(P.split, P.cf, q, split_sound<float>(P, a, 0, q), rm[s], rm[BOX + s], rm[2 * BOX + s],
                              rm[3 * BOX + s], rm[4 * BOX + s], rm[5 * BOX + s], rm[6 * BOX + s], fp, fm);
#pragma unroll
            for (int n = 0; n < 5; n++) {
                sFp[n * BOX + s] = fp[n];
                sFm[n * BOX + s] = fm[n];
            }
            sS[s] = rm[6 * BOX + s];
            if (hybrid) sPhi[s] = rphi[s];
        }
        __syncthreads();
        // the staging buffer is free: start the next tile's copies under Phases B and C
        if (threadIdx.x == 0) {
            const int next = (int)atomicAdd(ctr, 1u);
            counts[4] = next;
            if (next < ntiles) issue(next);
        }

        // ---- Phase B: faces t = 0..nc (between positions t+3 and t+4); WENO faces queued
        auto do_face = [&](int l, int t, int br) {
            const long long cl = cell(l, c0 + t + 3), cr = cl + stride;
            float out[5];
            const float s0f = (br == 1 || br == 2) ? 2.f / (sS[sidx(l, t + 3)] + sS[sidx(l, t + 4)]) : 0.f;
            auto FP = [&](int n, int p) { return sFp[n * BOX + sidx(l, p)]; };
            auto FM = [&](int n, int p) { return sFm[n * BOX + sidx(l, p)]; };
            face_flux<CHAR, float>(P, a, br, t, s0f, cl, cr, FP, FM, out);
            const int f = fidx(l, t);
#pragma unroll
            for (int n = 0; n < 5; n++) sF[n * TL * NF + f] = out[n];
        };
        for (int it = threadIdx.x; it < TL * NF; it += NT) {
            int l, t;
            if (DIR == 0) { l = it / NF; t = it - l * NF; } else { t = it / TL; l = it - t * TL; }
            if (l >= nl || t > nc) continue;
            int br = P.fixed_branch;
            if (hybrid) {
                float ph[6];
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
            for (int k = threadIdx.x; k < n7 + n5; k += NT) {
                const int it = k < n7 ? list7[k] : list5[k - n7];
                int l, t;
                if (DIR == 0) { l = it / NF; t = it - l * NF; } else { t = it / TL; l = it - t * TL; }
                do_face(l, t, k < n7 ? 1 : 2);
            }
        }
        __syncthreads();
        if constexpr (EPI) {
            // ---- Phase C from the staged boxes: wait for this tile's copies (bounded)
            int eto = 0;
            if (threadIdx.x == 0) {
                eto = !mbar_wait_bounded(ebar, parity, kWaitLimitNs);
                if (eto) {  // drain: this tile's Phase C copies and the next tile's staged inputs
                    atomicOr(a.kstat, 1u);
                    mbar_wait_bounded(ebar, parity, kWaitLimitNs);
                    if (counts[4] < ntiles) mbar_wait_bounded(bar, parity ^ 1u, kWaitLimitNs);
                }
            }
            if (__syncthreads_or(eto)) return;
            staged_epilogue(c0, l0, other, nc, nl);
            __syncthreads();  // sF, the lists and the staged boxes are rewritten by the next tile
            if (threadIdx.x == 0 && counts[4] < ntiles) issue_epi(counts[4]);
        } else {
            // the next tile's Phase C inputs into L2 while this tile finishes (last sweep only)
            if (a.out_mode == OUT_RHS || a.out_mode == OUT_STAGE) prefetch_epilogue(counts[4]);

            // ---- Phase C: differences, viscous terms and the accumulation of out_mode
            sweep_epilogue<DIR, TL, TC, NT, float>(a, sF, c0, l0, other, nc, nl, cell, fidx);
            __syncthreads();  // sF, sPhi and the lists are rewritten by the next tile
        }
        tile = counts[4];
    }
}

// ---- host side ---------------------------------------------------------------------------
namespace {

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

// rank-3 or rank-4 tensor (x, y, z[, n]) over the full grid with component stride cstride
// bytes; FP32 (esize 4) or FP64 (esize 8) elements
bool encode(CUtensorMap* map, const DevParams& P, const void* base, int ncomp, size_t cstride, const unsigned box[3],
            int esize = 4) {
    auto fn = encode_fn();
    if (!fn || !base) return false;
    const int rank = ncomp > 1 ? 4 : 3;
    cuuint64_t dims[4] = {(cuuint64_t)P.nxt, (cuuint64_t)P.nyt, (cuuint64_t)P.nzt, (cuuint64_t)ncomp};
    cuuint64_t strides[3] = {(cuuint64_t)P.nxt * esize, (cuuint64_t)P.nxt * P.nyt * esize, (cuuint64_t)cstride};
    cuuint32_t bdim[4] = {box[0], box[1], box[2], (cuuint32_t)ncomp};
    cuuint32_t estr[4] = {1, 1, 1, 1};
    CUresult r = fn(map, esize == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank,
                    const_cast<void*>(base), dims, strides, bdim, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

template <int DIR> void box_of(unsigned box[3]) {
    using L = TmaLayout<DIR>;
    if (DIR == 0) { box[0] = L::NP; box[1] = L::TL; box[2] = 1; }
    else if (DIR == 1) { box[0] = L::TL; box[1] = L::NP; box[2] = 1; }
    else { box[0] = L::TL; box[1] = 1; box[2] = L::NP; }
}

constexpr int kMaxDev = 32;
int g_blocks[kMaxDev][3][2] = {};  // resident blocks per SM x SMs, per device, direction, char flag

int g_blocks_epi[kMaxDev][2] = {};  // the same for the staged-epilogue zeta sweep

template <int DIR, bool CHAR, bool EPI> cudaError_t configure_one(int dev) {
    auto k = k_sweep_tma<DIR, CHAR, EPI>;
    constexpr size_t smem = TmaLayout<DIR, EPI>::total;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int per_sm = 0, nsm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, TTile<DIR>::NT, smem)) != cudaSuccess)
        return e;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    (EPI ? g_blocks_epi[dev][CHAR ? 1 : 0] : g_blocks[dev][DIR][CHAR ? 1 : 0]) = (per_sm > 0 ? per_sm : 1) * nsm;
    return cudaSuccess;
}

template <int DIR, bool CHAR, bool EPI>
cudaError_t launch_one(const SweepArgs& a, const SweepMaps& m, const EpiMaps& em, int dev, cudaStream_t st) {
    using L = TmaLayout<DIR, EPI>;
    const DevParams& P = a.P;
    const int Nd = DIR == 0 ? P.nx : (DIR == 1 ? P.ny : P.nz);
    const int Nl = DIR == 0 ? P.ny : P.nx;
    const int No = DIR == 2 ? P.ny : P.nz;
    const long long ntiles = (long long)((Nd + L::TC - 1) / L::TC) * ((Nl + L::TL - 1) / L::TL) * No;
    int blocks = EPI ? g_blocks_epi[dev][CHAR ? 1 : 0] : g_blocks[dev][DIR][CHAR ? 1 : 0];
    if (blocks <= 0) return cudaErrorNotReady;
    if (ntiles < blocks) blocks = (int)ntiles;
    k_sweep_tma<DIR, CHAR, EPI><<<blocks, TTile<DIR>::NT, L::total, st>>>(a, m, em);
    return cudaGetLastError();
}

}  // namespace

bool sweep_tma_usable(const DevParams& P) {
    return P.nxt % 4 == 0 && encode_fn() != nullptr && (long long)P.nx * P.ny * P.nz < (1ll << 31);
}

cudaError_t sweep_tma_configure() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    if ((e = configure_one<0, false, false>(dev)) != cudaSuccess) return e;
    if ((e = configure_one<0, true, false>(dev)) != cudaSuccess) return e;
    if ((e = configure_one<1, false, false>(dev)) != cudaSuccess) return e;
    if ((e = configure_one<1, true, false>(dev)) != cudaSuccess) return e;
    if ((e = configure_one<2, false, false>(dev)) != cudaSuccess) return e;
    if ((e = configure_one<2, true, false>(dev)) != cudaSuccess) return e;
    if ((e = configure_one<2, false, true>(dev)) != cudaSuccess) return e;
    return configure_one<2, true, true>(dev);
}

// Tensor maps of the three directions over the context's FP32 arrays: Q32 (6 planes of
// P.plane floats), the metric packs (7 planes b1 bytes apart each) and the sensor.
cudaError_t make_sweep_maps(const DevParams& P, const float* q32, const float* const pack[3], size_t pack_stride,
                            const float* phi, void* out3) {
    SweepMaps* out = static_cast<SweepMaps*>(out3);
    unsigned b[3][3];
    box_of<0>(b[0]);
    box_of<1>(b[1]);
    box_of<2>(b[2]);
    for (int d = 0; d < 3; d++) {
        if (!encode(&out[d].q, P, q32, kQVars, (size_t)P.plane * 4, b[d]) ||
            !encode(&out[d].m, P, pack[d], kMetVars, pack_stride, b[d]) ||
            !encode(&out[d].phi, P, phi, 1, 0, b[d]))
            return cudaErrorInvalidValue;
    }
    return cudaSuccess;
}

size_t sweep_maps_bytes() { return sizeof(SweepMaps) * 3; }
size_t epi_maps_bytes() { return sizeof(EpiMaps); }

// Phase C maps of the last (zeta) sweep: the FP32 direction sums acc, acc2 (5 planes of
// P.plane floats each), J and, when given, U and Un (5 planes of P.plane doubles).
cudaError_t make_epi_maps(const DevParams& P, const float* acc, const float* acc2, const double* J,
                          const double* U, const double* Un, void* out) {
    EpiMaps* m = static_cast<EpiMaps*>(out);
    using L = TmaLayout<2, true>;
    const unsigned box[3] = {(unsigned)L::TL, 1u, (unsigned)L::TC};
    const size_t p4 = (size_t)P.plane * 4, p8 = (size_t)P.plane * 8;
    if (!encode(&m->acc, P, acc, 5, p4, box) || !encode(&m->acc2, P, acc2, 5, p4, box) ||
        !encode(&m->J, P, J, 1, 0, box, 8))
        return cudaErrorInvalidValue;
    if (U && !encode(&m->U, P, U, 5, p8, box, 8)) return cudaErrorInvalidValue;
    if (Un && !encode(&m->Un, P, Un, 5, p8, box, 8)) return cudaErrorInvalidValue;
    return cudaSuccess;
}

cudaError_t launch_sweep_tma(int dir, const SweepArgs& a, const void* maps3, const void* epi, cudaStream_t st) {
    const SweepMaps* m = static_cast<const SweepMaps*>(maps3);
    static const EpiMaps none{};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDev) return cudaErrorInvalidDevice;
    const bool ch = a.P.character != 0;
    if (dir == 0) return ch ? launch_one<0, true, false>(a, m[0], none, dev, st) : launch_one<0, false, false>(a, m[0], none, dev, st);
    if (dir == 1) return ch ? launch_one<1, true, false>(a, m[1], none, dev, st) : launch_one<1, false, false>(a, m[1], none, dev, st);
    if (epi) {
        const EpiMaps& em = *static_cast<const EpiMaps*>(epi);
        return ch ? launch_one<2, true, true>(a, m[2], em, dev, st) : launch_one<2, false, true>(a, m[2], em, dev, st);
    }
    return ch ? launch_one<2, true, false>(a, m[2], none, dev, st) : launch_one<2, false, false>(a, m[2], none, dev, st);
}

}  // namespace f3d
