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
    int precision;       // F3D_PREC_FP64 or F3D_PREC_MIXED
    int fixed_branch;    // -1: per-face hybrid switch; 0..3: every face takes that branch
    // FP64 sensor thresholds as bit patterns: for phi >= 0 (or NaN) the comparison
    // phi < t of the reference equals bits(phi) < phib (thresholds <= 0 or NaN map to 0,
    // which no phi is below), so the branch needs no FP64 instruction
    unsigned long long phib[3];
    Cst<double> cd;
    Cst<float> cf;
    int lts;            // local time stepping: per-cell dt in the stage update
    int les;            // F3D_LES_* in the viscous fluxes
    BcDev bc[6];
    const double* prof[6];  // F3D_BC_INFLOW_PROFILE states (5 x Ta x Tb), borrowed
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

// utils.jl:2-30 c2Prim of one cell. q = (rho,u,v,w,p,T).
__device__ __forceinline__ void c2prim_cell(const DevParams& P, const double U[5], double q[6]) {
    double rho = fmax(U[0], P.eps_clamp);
    if (U[0] != U[0]) rho = U[0];  // Julia max propagates NaN
    double rinv = 1.0 / rho;
    double u = __dmul_rn(U[1], rinv), v = __dmul_rn(U[2], rinv), w = __dmul_rn(U[3], rinv);
    double ke = __dadd_rn(__dadd_rn(__dmul_rn(u, u), __dmul_rn(v, v)), __dmul_rn(w, w));
    double eraw = __dadd_rn(U[4], -__dmul_rn(__dmul_rn(0.5, rho), ke));
    double ei = fmax(eraw, P.eps_clamp);
    if (eraw != eraw) ei = eraw;
    double p = __dmul_rn(P.gm1, ei);
    double T = p / __dmul_rn(rho, P.rg);
    q[0] = rho; q[1] = u; q[2] = v; q[3] = w; q[4] = p; q[5] = T;
}

// The same recovery for the mixed-precision form: still FP64 (the pressure/temperature
// recovery from total energy stays FP64), with T = p (1/rho)(1/Rg) instead of a second
// division. FP64 divisions are ~10 FMA issue slots on GB300.
__device__ __forceinline__ void c2prim_cell_fast(const DevParams& P, const double U[5], double q[6]) {
    double rho = fmax(U[0], P.eps_clamp);
    if (U[0] != U[0]) rho = U[0];
    const double rinv = 1.0 / rho;
    const double u = U[1] * rinv, v = U[2] * rinv, w = U[3] * rinv;
    const double eraw = U[4] - 0.5 * rho * (u * u + v * v + w * w);
    double ei = fmax(eraw, P.eps_clamp);
    if (eraw != eraw) ei = eraw;
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
