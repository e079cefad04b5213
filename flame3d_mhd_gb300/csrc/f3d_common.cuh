// f3d_common.cuh — device-side parameters, indexing and per-cell physics shared by the
// Flame3D GB300 kernels.
//
// Layout: every field is the reference's Julia array (Nxt,Nyt,Nzt,nvar), column-major,
// i fastest; the 0-based linear index of (i,j,k,n) is i + Nxt*(j + Nyt*(k + Nzt*n)).
// Indices in this file are 0-based on the full (ghost-including) grid unless named
// "interior"; interior cell ii corresponds to full index ii + NG.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/flame3d_gpu.h"

namespace f3d {

constexpr int NG = 4;  // ghost layers (parse_mesh.jl:6); the stencils below assume 4

struct BcDev {
    int kind;
    double rho, u, v, w, p, T;  // Dirichlet state with T = p/(rho Rg)
    double t_wall;
};

// Gas and scheme constants in the arithmetic type of a kernel, derived once on the host.
template <class R> struct Cst {
    R gamma, grg, gm1, rg;
    R inv_gm1;   // 1/(gamma-1)
    R inv_2g;    // 1/(2 gamma)          (split.jl:54)
    R two_gm1;   // 2 (gamma-1)          (split.jl:55)
    R w2c;       // (3-gamma)/(2(gamma-1)) (split.jl:52)
    R c_s, t_s, cp, pr;
    R cp_pr;     // cp / Pr: heat conductivity per unit viscosity
    R phi1, phi2, phi3;
    R lin[7];
};

// Runtime constants of one context, passed to every kernel by value.
// Exact quotient of n < 2^32 by a divisor d > 1 fixed for the grid: q = mulhi64(M, n) with
// M = ceil(2^64 / d) (Lemire, Kaser and Kurz, "Faster remainder by direct computation",
// 2019). Cell indices are decomposed this way instead of with 64-bit / and %, which
// compile to long emulated sequences.
struct FastDiv {
    unsigned long long M;
    unsigned d;
};
inline FastDiv make_fastdiv(unsigned d) { return FastDiv{d > 1 ? ~0ull / d + 1ull : 0ull, d}; }
__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv& f) {
    return f.d > 1 ? (unsigned)__umul64hi(f.M, (unsigned long long)n) : n;
}
// t = a + na (b + nb c) -> (a, b, c) with na = fa.d, nb = fb.d
__device__ __forceinline__ void split3(long long t, const FastDiv& fa, const FastDiv& fb, int& a, int& b, int& c) {
    const unsigned tu = (unsigned)t;
    const unsigned q = fdiv(tu, fa);
    a = (int)(tu - q * fa.d);
    const unsigned q2 = fdiv(q, fb);
    b = (int)(q - q2 * fb.d);
    c = (int)q2;
}

struct DevParams {
    int nx, ny, nz;     // interior
    int nxt, nyt, nzt;  // with ghosts
    long long plane;    // nxt*nyt*nzt
    double gamma, rg, cp, c_s, t_s, pr;
    double gm1;          // gamma - 1
    double inv_rg;       // 1 / Rg
    double grg;          // gamma * Rg (split.jl:22)
    double eps_clamp;    // utils.jl:12,18
    double phi1, phi2, phi3;
    double lin[7];       // run.jl:75-77
    int split, character, viscous;
    int precision;       // F3D_PREC_*
    int ref32;           // F3D_PREC_REF32: Float32 arrays and the reference's Float32 arithmetic
    float g32, rg32, gm1_32, eps32;  // its Float32 constants: gamma, Rg, gamma - 1, the clamp
    int fixed_branch;    // -1: per-face hybrid switch; 0..3: every face takes that branch
    // FP64 sensor thresholds as bit patterns: for phi >= 0 (or NaN) the comparison
    // phi < t of the reference equals bits(phi) < phib (thresholds <= 0 or NaN map to 0,
    // which no phi is below), so the branch needs no FP64 instruction
    unsigned long long phib[3];
    Cst<double> cd;
    Cst<float> cf;
    FastDiv dnxt, dnyt;  // full-grid extents: cell index -> (i, j, k)
    FastDiv dnx, dny;    // interior extents
    FastDiv dvxt, dvyt;  // the viscous box (Nt - 4 per direction)
    int lts;            // local time stepping: per-cell dt in the stage update
    int les;            // F3D_LES_* in the viscous fluxes
    BcDev bc[6];
    const double* prof[6];  // F3D_BC_INFLOW_PROFILE states (5 x Ta x Tb), borrowed
    double* profb[6];       // their cotangents, accumulated by the adjoint when set
};

template <class R> __host__ __device__ inline const Cst<R>& cst(const DevParams& P);
template <> __host__ __device__ inline const Cst<double>& cst<double>(const DevParams& P) { return P.cd; }
template <> __host__ __device__ inline const Cst<float>& cst<float>(const DevParams& P) { return P.cf; }

__host__ __device__ inline long long lin3(const DevParams& P, int i, int j, int k) {
    return (long long)i + (long long)P.nxt * ((long long)j + (long long)P.nyt * k);
}

// ------------------------------------------------------------------------------------
// Per-cell physics in FP64 with the reference's operation order. __dmul_rn/__dadd_rn
// keep nvcc from contracting into FMA so that c2Prim and the ghost rules are bitwise
// equal to the CPU restatement; the flux arithmetic is free to contract.

// Julia's max(x, e) (a NaN x passes through) for a floor e > 0, on the bit patterns with
// integer instructions instead of FP64-pipe compares: for x >= 0 the order of doubles is the
// integer order of their patterns, a negative x (sign bit set) is a negative integer, and a
// NaN has all exponent bits set and a nonzero mantissa. The same value as fmax for every x.
__device__ __forceinline__ double max_floor(double x, double e) {
    const long long bx = __double_as_longlong(x), be = __double_as_longlong(e);
    if (be <= 0) return x != x ? x : fmax(x, e);  // a floor of 0 or below
    return (bx > be || (bx & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL) ? x : e;
}

// utils.jl:2-30 c2Prim of one cell. q = (rho,u,v,w,p,T).
__device__ __forceinline__ void c2prim_cell(const DevParams& P, const double U[5], double q[6]) {
    const double rho = max_floor(U[0], P.eps_clamp);
    double rinv = 1.0 / rho;
    double u = __dmul_rn(U[1], rinv), v = __dmul_rn(U[2], rinv), w = __dmul_rn(U[3], rinv);
    double ke = __dadd_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)), __dmul_rn(w, w));
    double eraw = __dadd_rn(U[4], -__dmul_rn(__dmul_rn(0.5, rho), ke));
    const double ei = max_floor(eraw, P.eps_clamp);
    double p = __dmul_rn(P.gm1, ei);
    double T = p / __dmul_rn(rho, P.rg);
    q[0] = rho; q[1] = u; q[2] = v; q[3] = w; q[4] = p; q[5] = T;
}

// The same recovery for the mixed-precision form: still FP64 (the pressure/temperature
// recovery from total energy stays FP64), with 1/rho by recip_nr and T = p (1/rho)(1/Rg)
// instead of divisions: FP64 divisions are ~10 FMA issue slots on GB300.
// ---- conversions and a reciprocal for the mixed form, off the FP64 pipe -----------------
// On this GPU the double <-> float conversion instructions issue on the FP64 pipe, which
// the mixed form needs for its FP64 state arithmetic. These work on the IEEE 754 binary64 /
// binary32 bit layouts with integer operations in the binary32 normal range and use the
// conversion instruction elsewhere (zeros, subnormal results, overflow, infinities, NaN).
__device__ __forceinline__ float f64_to_f32_rn(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned int hi = (unsigned int)(b >> 32);
    const int e = (int)((hi >> 20) & 0x7ffu);  // biased binary64 exponent
    if (e < 897 || e > 1150) return __double2float_rn(x);  // outside binary32 exponents 1..254
    const unsigned int m23 = (unsigned int)((b >> 29) & 0x7fffffull);
    const unsigned int rest = (unsigned int)(b & 0x1fffffffull);  // the 29 dropped bits
    unsigned int f = (hi & 0x80000000u) | ((unsigned int)(e - 896) << 23) | m23;
    // round to nearest, ties to even; a carry out of the mantissa moves to the next binade
    // (and from the largest finite binade to infinity), as rounding requires
    if (rest > 0x10000000u || (rest == 0x10000000u && (m23 & 1u))) f += 1u;
    return __uint_as_float(f);
}
__device__ __forceinline__ double f32_to_f64(float x) {  // exact
    const unsigned int b = __float_as_uint(x);
    const unsigned int e = (b >> 23) & 0xffu;
    if (e == 0u || e == 0xffu) return (double)x;
    const unsigned long long r = ((unsigned long long)(b & 0x80000000u) << 32) |
                                 ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)(b & 0x7fffffu) << 29);
    return __longlong_as_double((long long)r);
}
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) { return f32_to_f64(x); }

// 1/x: an FP32 reciprocal refined by two Newton-Raphson steps r <- r + r (1 - x r) in FP64
// (quadratic convergence from 2^-24 to below FP64 rounding), within an ulp of the FP64
// quotient; IEEE division outside 2^-119 <= |x| < 2^120 (and for 0, infinities and NaN).
__device__ __forceinline__ double recip_nr(double x) {
    // the range test on the biased exponent (integer instructions): 2^-119 <= |x| < 2^120
    const unsigned ex = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
    if (ex - 904u > 238u) return 1.0 / x;
    double r = f32_to_f64(__frcp_rn(f64_to_f32_rn(x)));
    r = fma(r, fma(-x, r, 1.0), r);
    return fma(r, fma(-x, r, 1.0), r);
}

__device__ __forceinline__ void c2prim_cell_fast(const DevParams& P, const double U[5], double q[6]) {
    const double rho = max_floor(U[0], P.eps_clamp);
    const double rinv = recip_nr(rho);
    const double u = U[1] * rinv, v = U[2] * rinv, w = U[3] * rinv;
    // rho |u|^2 / 2 as (momentum . velocity) / 2, folded into the subtraction from E
    const double eraw = fma(-0.5, U[1] * u + U[2] * v + U[3] * w, U[4]);
    const double ei = max_floor(eraw, P.eps_clamp);
    const double p = P.gm1 * ei;
    q[0] = rho; q[1] = u; q[2] = v; q[3] = w; q[4] = p; q[5] = p * (rinv * P.inv_rg);
}

// utils.jl:33-54 prim2c of one cell (also the U of Dirichlet and wall ghosts,
// boundary.jl:33-37, 88-92).
__device__ __forceinline__ void prim2c_cell(const DevParams& P, const double q[6], double U[5]) {
    double ei = q[4] / P.gm1;
    U[0] = q[0];
    U[1] = __dmul_rn(q[1], q[0]);
    U[2] = __dmul_rn(q[2], q[0]);
    U[3] = __dmul_rn(q[3], q[0]);
    double ke = __dadd_rn(__dadd_rn(__dmul_rn(q[1], q[1]), __dmul_rn(q[2], q[2])), __dmul_rn(q[3], q[3]));
    U[4] = __dadd_rn(ei, __dmul_rn(__dmul_rn(0.5, q[0]), ke));
}

// ------------------------------------------------------------------------------------
// Ghost rules. A ghost cell's final value is written by the last of the passes x, y, z
// that covers it (boundary.jl:151-156 order). resolve_ghost walks the passes from z back
// to x, moving the location through copy rules and recording the value transforms, so
// one thread can produce the cell's final value from one interior source cell.
struct GhostChain {
    int si, sj, sk;     // interior source cell (full index)
    int dirichlet;      // >= 0: the chain ends in the Dirichlet state of that face
    int nmirror;        // number of wall mirrors applied (velocity sign flips)
    int iso_face;       // last isothermal wall face applied, -1 if none
    bool nontrivial;    // a wall or Dirichlet rule is in the chain (U ghost = prim2c(Q))
    long long poff, pst; // inflow-profile chains: transverse offset and plane size
};

__device__ __forceinline__ int ghost_src(int kind, bool high, int g, int N) {
    // g, N are 0-based full index and interior count along the direction
    if (kind == F3D_BC_PERIODIC) return high ? g - N : g + N;                       // mpi.jl:105-282
    if (kind == F3D_BC_ZERO_GRADIENT) return high ? N + NG - 1 : NG;                // boundary.jl:43
    if (kind == F3D_BC_WALL_ADIABATIC || kind == F3D_BC_WALL_ISOTHERMAL)
        return high ? 2 * (N + NG) - 1 - g : 2 * NG - 1 - g;                        // boundary.jl:69
    return g;
}

__device__ __forceinline__ GhostChain resolve_ghost(const DevParams& P, int i, int j, int k) {
    GhostChain c;
    c.poff = 0;
    c.pst = 0;
    c.dirichlet = -1;
    c.nmirror = 0;
    c.iso_face = -1;
    c.nontrivial = false;
    int idx[3] = {i, j, k};
    const int N[3] = {P.nx, P.ny, P.nz};
    // Walk z, y, x (reverse fill order). Isothermal walls are only composed with copy
    // rules (a second transform would need the chain of two non-linear maps); the
    // parameter validation rejects isothermal walls on more than one direction.
    for (int d = 2; d >= 0; d--) {
        const int g = idx[d];
        const bool lo = g < NG, hi = g >= N[d] + NG;
        if (!lo && !hi) continue;
        const BcDev& b = P.bc[2 * d + (hi ? 1 : 0)];
        if (b.kind == F3D_BC_DIRICHLET || b.kind == F3D_BC_INFLOW_PROFILE) {
            c.dirichlet = 2 * d + (hi ? 1 : 0);
            c.nontrivial = true;
            if (b.kind == F3D_BC_INFLOW_PROFILE) {
                // transverse point where the chain reaches this face's pass
                const int a = d == 0 ? idx[1] : idx[0], bb = d == 2 ? idx[1] : idx[2];
                const long long ta = d == 0 ? P.nyt : P.nxt, tb = d == 2 ? P.nyt : P.nzt;
                c.poff = a + ta * bb;
                c.pst = ta * tb;
            }
            break;
        }
        if (b.kind == F3D_BC_WALL_ADIABATIC || b.kind == F3D_BC_WALL_ISOTHERMAL) {
            c.nmirror++;
            c.nontrivial = true;
            if (b.kind == F3D_BC_WALL_ISOTHERMAL && c.iso_face < 0) c.iso_face = 2 * d + (hi ? 1 : 0);
        }
        idx[d] = ghost_src(b.kind, hi, g, N[d]);
    }
    c.si = idx[0];
    c.sj = idx[1];
    c.sk = idx[2];
    return c;
}

// Apply the transforms of a chain to the source primitive state q (in place).
// The walk records the outermost rules first; the values are produced innermost first:
// Dirichlet state (if any), then mirrors. Velocity flips commute with each other, and
// an isothermal rule is the outermost non-copy rule by construction.
__device__ __forceinline__ void apply_chain(const DevParams& P, const GhostChain& c, double q[6]) {
    if (c.dirichlet >= 0) {
        const BcDev& b = P.bc[c.dirichlet];
        if (b.kind == F3D_BC_INFLOW_PROFILE) {
            const double* pr = P.prof[c.dirichlet] + c.poff;
            q[0] = pr[0]; q[1] = pr[c.pst]; q[2] = pr[2 * c.pst]; q[3] = pr[3 * c.pst]; q[4] = pr[4 * c.pst];
            q[5] = q[4] / __dmul_rn(q[0], P.rg);
        } else {
            q[0] = b.rho; q[1] = b.u; q[2] = b.v; q[3] = b.w; q[4] = b.p; q[5] = b.T;
        }
    }
    if (c.nmirror & 1) {
        q[1] = -q[1];
        q[2] = -q[2];
        q[3] = -q[3];
    }
    if (c.iso_face >= 0) {
        q[5] = __dadd_rn(__dmul_rn(2.0, P.bc[c.iso_face].t_wall), -q[5]);
        q[0] = q[4] / __dmul_rn(P.rg, q[5]);
    }
}

// ------------------------------------------------------------------------------------
// Small helpers
template <class T> __device__ __forceinline__ T sq(T a) { return a * a; }
template <class T> __device__ __forceinline__ T minmod(T a, T b) {
    return (a * b > T(0)) ? ((fabs(a) > fabs(b)) ? b : a) : T(0);
}

inline unsigned cdiv(long long a, long long b) { return (unsigned)((a + b - 1) / b); }

}  // namespace f3d
