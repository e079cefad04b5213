// f3d_oracle.hpp — CPU restatement of the Flame3D finite-difference RHS and SSP-RK3 stage.
//
// TEST INFRASTRUCTURE ONLY. This is the oracle the CUDA library is checked against; it
// is built and called by tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline
// leg, never by the library itself.
//
// Every function restates one reference kernel (file:line given beside it) with the same
// formulas, the same operation order and the same index ranges. Indices are 1-based like
// the reference's Julia arrays so each line can be read against the source. Arrays keep
// the reference layout (Nxt, Nyt, Nzt, nvar) column-major, i fastest.
//
// Template parameters: R is the working type; W is the type of the WENO7 nonlinear
// weights. <double,double> is the FP64 oracle. <float,double> mirrors the reference's own
// arithmetic: Float32 everywhere except the WENO7 alphas, which the reference promotes to
// Float64 through `WENOϵ1::Float64 = 1e-20` (schemes.jl:98, :712). The reference launches
// with fastmath=true; the <float,double> instantiation uses IEEE operations instead.
//
// Parity is unpinned by the reference's own tests: the reference has no tests, fixtures
// or golden vectors, and Julia is not available to run it. The one piece of the reference
// that runs here, its Python coefficient script (Utils/FDMcoeffs.py), pins the UP7 and CD6
// face coefficients (tests/golden/fdm_coeffs.json).
#pragma once
#include <type_traits>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "../include/flame3d_gpu.h"

namespace f3do {

using std::abs;
using std::sqrt;
using std::cbrt;
using std::pow;

// NaN-propagating max/min like Julia's max/min on floats.
template <class T> inline T jmax(const T& a, const T& b) {
    if (a != a) return a;
    if (b != b) return b;
    return (a < b) ? b : a;
}
template <class T> inline T jmin(const T& a, const T& b) {
    if (a != a) return a;
    if (b != b) return b;
    return (b < a) ? b : a;
}
template <class T> inline T sq(const T& a) { return a * a; }

// minmod, schemes.jl:26-28
template <class T> inline T minmod(const T& a, const T& b) {
    return (a * b > T(0)) ? ((abs(a) > abs(b)) ? b : a) : T(0);
}

// Grid with the reference's sizes: interior N, ghosts NG, totals N + 2NG.
struct Grid {
    long nx, ny, nz, ng, nxt, nyt, nzt;
    explicit Grid(const f3d_params& p)
        : nx(p.nx), ny(p.ny), nz(p.nz), ng(p.ng), nxt(p.nx + 2 * p.ng),
          nyt(p.ny + 2 * p.ng), nzt(p.nz + 2 * p.ng) {}
    size_t ncell() const { return (size_t)nxt * nyt * nzt; }
    long n(int d) const { return d == 0 ? nx : (d == 1 ? ny : nz); }
    long nt(int d) const { return d == 0 ? nxt : (d == 1 ? nyt : nzt); }
    long stride(int d) const { return d == 0 ? 1 : (d == 1 ? nxt : nxt * nyt); }
};

// Non-owning view of a column-major 4-D array with 1-based indexing.
template <class T> struct V4 {
    T* p;
    long n1, n2, n3;
    T& operator()(long i, long j, long k, long n = 1) const {
        return p[(i - 1) + n1 * ((j - 1) + n2 * ((k - 1) + n3 * (n - 1)))];
    }
    size_t lin(long i, long j, long k) const { return (size_t)((i - 1) + n1 * ((j - 1) + n2 * (k - 1))); }
    size_t plane() const { return (size_t)n1 * n2 * n3; }
};

// Scalar constants of one instantiation (run.jl:8-13, 70-77; schemes.jl:95-107).
template <class R> struct Consts {
    R gamma, rg, cp, c_s, t_s, pr, phi1, phi2, phi3, eps_clamp;
    R lin[7];
    explicit Consts(const f3d_params& p) {
        gamma = R(p.gamma);
        rg = R(p.rg);
        cp = p.cp != 0.0 ? R(p.cp) : rg * gamma / (gamma - R(1));
        c_s = R(p.c_s);
        t_s = R(p.t_s);
        pr = R(p.pr);
        phi1 = R(p.phi1);
        phi2 = R(p.phi2);
        phi3 = R(p.phi3);
        eps_clamp = R(p.clamp_eps != 0.0 ? p.clamp_eps : 1.1920928955078125e-07);
        // run.jl:75-77: Linear = UP7*Linear_ϕ + CD6*(1-Linear_ϕ)
        const double up7[7] = {-3.0 / 420, 25.0 / 420, -101.0 / 420, 319.0 / 420,
                               214.0 / 420, -38.0 / 420, 4.0 / 420};
        const double cd6[7] = {0.0, 1.0 / 60, -2.0 / 15, 37.0 / 60, 37.0 / 60, -2.0 / 15, 1.0 / 60};
        R lp = R(p.linear_phi);
        for (int m = 0; m < 7; m++) lin[m] = R(up7[m]) * lp + R(cd6[m]) * (R(1) - lp);
    }
};

// ---------------------------------------------------------------------------------
// utils.jl:2-30 c2Prim — interior cells, clamps on rho and e_int.
template <class R> void c2prim(const f3d_params& P, const R* Up, R* Qp) {
    Grid g(P);
    Consts<R> C(P);
    V4<const R> U{Up, g.nxt, g.nyt, g.nzt};
    V4<R> Q{Qp, g.nxt, g.nyt, g.nzt};
    const long NG = g.ng;
#pragma omp parallel for schedule(static)
    for (long k = NG + 1; k <= g.nz + NG; k++)
        for (long j = NG + 1; j <= g.ny + NG; j++)
            for (long i = NG + 1; i <= g.nx + NG; i++) {
                R rho = jmax(U(i, j, k, 1), C.eps_clamp);
                R rinv = R(1) / rho;
                R u = U(i, j, k, 2) * rinv;
                R v = U(i, j, k, 3) * rinv;
                R w = U(i, j, k, 4) * rinv;
                R ei = jmax(U(i, j, k, 5) - R(0.5) * rho * (u * u + v * v + w * w), C.eps_clamp);
                R p = (C.gamma - R(1)) * ei;
                R T = p / (rho * C.rg);
                Q(i, j, k, 1) = rho;
                Q(i, j, k, 2) = u;
                Q(i, j, k, 3) = v;
                Q(i, j, k, 4) = w;
                Q(i, j, k, 5) = p;
                Q(i, j, k, 6) = T;
            }
}

// utils.jl:33-54 prim2c — every cell.
template <class R> inline void prim2c_cell(const Consts<R>& C, R rho, R u, R v, R w, R p, R out[5]) {
    R ei = p / (C.gamma - R(1));
    out[0] = rho;
    out[1] = u * rho;
    out[2] = v * rho;
    out[3] = w * rho;
    out[4] = ei + R(0.5) * rho * (u * u + v * v + w * w);
}
template <class R> void prim2c(const f3d_params& P, const R* Qp, R* Up) {
    Grid g(P);
    Consts<R> C(P);
    V4<const R> Q{Qp, g.nxt, g.nyt, g.nzt};
    V4<R> U{Up, g.nxt, g.nyt, g.nzt};
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= g.nzt; k++)
        for (long j = 1; j <= g.nyt; j++)
            for (long i = 1; i <= g.nxt; i++) {
                R o[5];
                prim2c_cell(C, Q(i, j, k, 1), Q(i, j, k, 2), Q(i, j, k, 3), Q(i, j, k, 4),
                            Q(i, j, k, 5), o);
                for (int n = 0; n < 5; n++) U(i, j, k, n + 1) = o[n];
            }
}

// utils.jl:57-70 linComb — interior cells.
template <class R> void lincomb(const f3d_params& P, R* Up, const R* Unp, R a, R b) {
    Grid g(P);
    V4<R> U{Up, g.nxt, g.nyt, g.nzt};
    V4<const R> Un{Unp, g.nxt, g.nyt, g.nzt};
    const long NG = g.ng;
#pragma omp parallel for schedule(static)
    for (long k = NG + 1; k <= g.nz + NG; k++)
        for (long n = 1; n <= 5; n++)
            for (long j = NG + 1; j <= g.ny + NG; j++)
                for (long i = NG + 1; i <= g.nx + NG; i++) U(i, j, k, n) = U(i, j, k, n) * a + Un(i, j, k, n) * b;
}

// The Dirichlet ghost state (rho, u, v, w, p) with T = p / (rho Rg) and its conserved form.
template <class R>
void set_dirichlet(const Consts<R>& C, R rho, R u, R v, R w, R p, V4<R>& Q, V4<R>& U, long gi, long gj, long gk) {
    R T = p / (rho * C.rg);
    Q(gi, gj, gk, 1) = rho;
    Q(gi, gj, gk, 2) = u;
    Q(gi, gj, gk, 3) = v;
    Q(gi, gj, gk, 4) = w;
    Q(gi, gj, gk, 5) = p;
    Q(gi, gj, gk, 6) = T;
    U(gi, gj, gk, 1) = rho;
    U(gi, gj, gk, 2) = rho * u;
    U(gi, gj, gk, 3) = rho * v;
    U(gi, gj, gk, 4) = rho * w;
    U(gi, gj, gk, 5) = p / (C.gamma - R(1)) + R(0.5) * rho * (u * u + v * v + w * w);
}

// A value of type R seeded with a tangent: only dual numbers carry it.
template <class R> inline R seeded(double v, double) { return R(v); }
template <> inline Dual seeded<Dual>(double v, double d) { return Dual(v, d); }

// ---------------------------------------------------------------------------------
// Ghost fill: mpi.jl:2-103 (periodic exchange with self) and boundary.jl:1-156
// (fill_x, fill_y, fill_z), applied in the order x, y, z over the full transverse
// extent including ghosts. Each face rule writes Q (6 vars) and U (5 vars).
template <class R>
void fill_ghost_cell(const f3d_params& P, const Consts<R>& C, const f3d_bc& bc, V4<R>& Q, V4<R>& U,
                     long gi, long gj, long gk, long si, long sj, long sk) {
    switch (bc.kind) {
    case F3D_BC_PERIODIC:
    case F3D_BC_ZERO_GRADIENT:  // boundary.jl:42-51, mpi.jl pack/unpack
        for (int n = 1; n <= 6; n++) Q(gi, gj, gk, n) = Q(si, sj, sk, n);
        for (int n = 1; n <= 5; n++) U(gi, gj, gk, n) = U(si, sj, sk, n);
        break;
    case F3D_BC_DIRICHLET:  // boundary.jl:12-38 and 98-118
        set_dirichlet(C, R(bc.rho), R(bc.u), R(bc.v), R(bc.w), R(bc.p), Q, U, gi, gj, gk);
        break;
    case F3D_BC_WALL_ADIABATIC:
    case F3D_BC_WALL_ISOTHERMAL: {  // boundary.jl:67-93 (mirror about the wall)
        R rho = Q(si, sj, sk, 1), p = Q(si, sj, sk, 5), T = Q(si, sj, sk, 6);
        R u = -Q(si, sj, sk, 2), v = -Q(si, sj, sk, 3), w = -Q(si, sj, sk, 4);
        if (bc.kind == F3D_BC_WALL_ISOTHERMAL) {
            T = R(2) * R(bc.t_wall) - T;
            rho = p / (C.rg * T);
        }
        Q(gi, gj, gk, 1) = rho;
        Q(gi, gj, gk, 5) = p;
        Q(gi, gj, gk, 6) = T;
        Q(gi, gj, gk, 2) = u;
        Q(gi, gj, gk, 3) = v;
        Q(gi, gj, gk, 4) = w;
        U(gi, gj, gk, 1) = rho;
        U(gi, gj, gk, 2) = rho * u;
        U(gi, gj, gk, 3) = rho * v;
        U(gi, gj, gk, 4) = rho * w;
        U(gi, gj, gk, 5) = p / (C.gamma - R(1)) + R(0.5) * rho * (u * u + v * v + w * w);
        break;
    }
    default:
        break;
    }
}

// Per-point inflow states of F3D_BC_INFLOW_PROFILE faces (5 x Ta x Tb doubles each, the
// layout of f3d_set_inflow_profile), registered by orc_set_inflow_profile.
inline const double*& inflow_profile(int face) {
    static const double* prof[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    return prof[face];
}

// Optional tangent of an inflow profile (same layout): dual-number runs seed the profile's
// ghost states with it (forward-mode derivative with respect to the profile).
inline const double*& inflow_profile_tangent(int face) {
    static const double* dprof[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    return dprof[face];
}

// Cell-centre coordinates (x, y, z with ghosts) for the finite-volume schemes, registered
// by orc_set_coordinates; every Solver of a finite-volume scheme copies them in its type.
inline const double** coordinates() {
    static const double* xyz[3] = {nullptr, nullptr, nullptr};
    return xyz;
}

// Source layer (1-based index along the direction) of ghost layer g for a face rule.
inline long ghost_source(int kind, bool high, long g, long N, long NG) {
    if (kind == F3D_BC_PERIODIC) return high ? g - N : g + N;           // mpi.jl:105-282
    if (kind == F3D_BC_ZERO_GRADIENT) return high ? N + NG : NG + 1;    // boundary.jl:43
    if (kind == F3D_BC_WALL_ADIABATIC || kind == F3D_BC_WALL_ISOTHERMAL)
        return high ? 2 * (N + NG) + 1 - g : 2 * NG + 1 - g;            // boundary.jl:69
    return g;                                                           // Dirichlet: unused
}

template <class R> void fill_ghosts(const f3d_params& P, R* Qp, R* Up) {
    Grid g(P);
    Consts<R> C(P);
    V4<R> Q{Qp, g.nxt, g.nyt, g.nzt};
    V4<R> U{Up, g.nxt, g.nyt, g.nzt};
    const long NG = g.ng;
    for (int d = 0; d < 3; d++) {
        const long N = g.n(d);
        for (int side = 0; side < 2; side++) {
            const f3d_bc& bc = P.bc[2 * d + side];
            const bool high = side == 1;
            const long g0 = high ? N + NG + 1 : 1, g1 = high ? N + 2 * NG : NG;
            // the two transverse extents (full, including ghosts)
            const long ta = d == 0 ? g.nyt : g.nxt;
            const long tb = d == 2 ? g.nyt : g.nzt;
#pragma omp parallel for schedule(static)
            for (long b = 1; b <= tb; b++)
                for (long a = 1; a <= ta; a++)
                    for (long gg = g0; gg <= g1; gg++) {
                        long s = ghost_source(bc.kind, high, gg, N, NG);
                        long gi, gj, gk, si, sj, sk;
                        if (d == 0) { gi = gg; gj = a; gk = b; si = s; sj = a; sk = b; }
                        else if (d == 1) { gi = a; gj = gg; gk = b; si = a; sj = s; sk = b; }
                        else { gi = a; gj = b; gk = gg; si = a; sj = b; sk = s; }
                        if (bc.kind == F3D_BC_INFLOW_PROFILE) {
                            // the inlet of boundary.jl:10-38 with the state of this point
                            const double* pr = inflow_profile(2 * d + side);
                            const double* dp = inflow_profile_tangent(2 * d + side);
                            const long st = ta * tb, off = (a - 1) + ta * (b - 1);
                            R q[5];
                            for (int n = 0; n < 5; n++)  // not registered: NaN ghosts, for the caller to see
                                q[n] = seeded<R>(pr ? pr[off + n * st] : std::numeric_limits<double>::quiet_NaN(),
                                                 dp ? dp[off + n * st] : 0.0);
                            set_dirichlet(C, q[0], q[1], q[2], q[3], q[4], Q, U, gi, gj, gk);
                            continue;
                        }
                        fill_ghost_cell(P, C, bc, Q, U, gi, gj, gk, si, sj, sk);
                    }
        }
    }
}

// ---------------------------------------------------------------------------------
// schemes.jl:1-24 shockSensor — cells 2..Nt-1 in every direction.
template <class R> void sensor(const f3d_params& P, const R* Qp, R* phip) {
    Grid g(P);
    V4<const R> Q{Qp, g.nxt, g.nyt, g.nzt};
    V4<R> phi{phip, g.nxt, g.nyt, g.nzt};
#pragma omp parallel for schedule(static)
    for (long k = 2; k <= g.nzt - 1; k++)
        for (long j = 2; j <= g.nyt - 1; j++)
            for (long i = 2; i <= g.nxt - 1; i++) {
                R px1 = Q(i - 1, j, k, 5), px2 = Q(i, j, k, 5), px3 = Q(i + 1, j, k, 5);
                R py1 = Q(i, j - 1, k, 5), py2 = Q(i, j, k, 5), py3 = Q(i, j + 1, k, 5);
                R pz1 = Q(i, j, k - 1, 5), pz2 = Q(i, j, k, 5), pz3 = Q(i, j, k + 1, 5);
                R fx = abs(-px1 + R(2) * px2 - px3) / (px1 + R(2) * px2 + px3);
                R fy = abs(-py1 + R(2) * py2 - py3) / (py1 + R(2) * py2 + py3);
                R fz = abs(-pz1 + R(2) * pz2 - pz3) / (pz1 + R(2) * pz2 + pz3);
                phi(i, j, k) = fx + fy + fz;
            }
}

// ---------------------------------------------------------------------------------
// Flux-vector splitting at one cell. q = (rho,u,v,w,p,T); A = metric row of the
// direction (J^-1-scaled); ss = |A|. Writes fp[5], fm[5].
template <class R>
void split_cell(int method, const Consts<R>& C, const R q[6], R A1, R A2, R A3, R ss, R fp[5], R fm[5]) {
    const R g = C.gamma;
    const R rho = q[0], u = q[1], v = q[2], w = q[3], p = q[4], T = q[5];
    if (method == F3D_SPLIT_SW) {  // split.jl:2-68
        R c = sqrt(g * C.rg * T);
        R E1 = A1 * u + A2 * v + A3 * w;
        R E2 = E1 - c * ss;
        R E3 = E1 + c * ss;
        R sinv = R(1) / ss;
        A1 = A1 * sinv;
        A2 = A2 * sinv;
        A3 = A3 * sinv;
        R E1P = (E1 + abs(E1)) * R(0.5);
        R E2P = (E2 + abs(E2)) * R(0.5);
        R E3P = (E3 + abs(E3)) * R(0.5);
        R E1M = E1 - E1P;
        R E2M = E2 - E2P;
        R E3M = E3 - E3P;
        R uc1 = u - c * A1, uc2 = u + c * A1;
        R vc1 = v - c * A2, vc2 = v + c * A2;
        R wc1 = w - c * A3, wc2 = w + c * A3;
        R vvc1 = (uc1 * uc1 + vc1 * vc1 + wc1 * wc1) * R(0.5);
        R vvc2 = (uc2 * uc2 + vc2 * vc2 + wc2 * wc2) * R(0.5);
        R vv = (g - R(1)) * (u * u + v * v + w * w);
        R W2 = (R(3) - g) / (R(2) * (g - R(1))) * (c * c);
        R t1 = rho / (R(2) * g);
        R t2 = R(2) * (g - R(1));
        fp[0] = t1 * (t2 * E1P + E2P + E3P);
        fp[1] = t1 * (t2 * E1P * u + E2P * uc1 + E3P * uc2);
        fp[2] = t1 * (t2 * E1P * v + E2P * vc1 + E3P * vc2);
        fp[3] = t1 * (t2 * E1P * w + E2P * wc1 + E3P * wc2);
        fp[4] = t1 * (E1P * vv + E2P * vvc1 + E3P * vvc2 + W2 * (E2P + E3P));
        fm[0] = t1 * (t2 * E1M + E2M + E3M);
        fm[1] = t1 * (t2 * E1M * u + E2M * uc1 + E3M * uc2);
        fm[2] = t1 * (t2 * E1M * v + E2M * vc1 + E3M * vc2);
        fm[3] = t1 * (t2 * E1M * w + E2M * wc1 + E3M * wc2);
        fm[4] = t1 * (E1M * vv + E2M * vvc1 + E3M * vvc2 + W2 * (E2M + E3M));
    } else if (method == F3D_SPLIT_LF) {  // split.jl:70-108
        R c = sqrt(g * p / rho);
        R un = A1 * u + A2 * v + A3 * w;
        R l0 = abs(un) + c * ss;
        R E0 = p / (g - R(1)) + R(0.5) * rho * (u * u + v * v + w * w);
        fp[0] = R(0.5) * (rho * un + l0 * rho);
        fp[1] = R(0.5) * (rho * u * un + A1 * p + l0 * rho * u);
        fp[2] = R(0.5) * (rho * v * un + A2 * p + l0 * rho * v);
        fp[3] = R(0.5) * (rho * w * un + A3 * p + l0 * rho * w);
        fp[4] = R(0.5) * ((E0 + p) * un + l0 * E0);
        fm[0] = R(0.5) * (rho * un - l0 * rho);
        fm[1] = R(0.5) * (rho * u * un + A1 * p - l0 * rho * u);
        fm[2] = R(0.5) * (rho * v * un + A2 * p - l0 * rho * v);
        fm[3] = R(0.5) * (rho * w * un + A3 * p - l0 * rho * w);
        fm[4] = R(0.5) * ((E0 + p) * un - l0 * E0);
    } else if (method == F3D_SPLIT_VL || method == F3D_SPLIT_AUSM) {
        R c = sqrt(g * p / rho);
        R un = A1 * u + A2 * v + A3 * w;
        R M = un / (c * ss);
        R full[5];
        if (method == F3D_SPLIT_VL) {  // split.jl:110-183
            R E0 = p / (g - R(1)) + R(0.5) * rho * (u * u + v * v + w * w);
            full[0] = rho * un;
            full[1] = rho * u * un + A1 * p;
            full[2] = rho * v * un + A2 * p;
            full[3] = rho * w * un + A3 * p;
            full[4] = (E0 + p) * un;
            if (M <= R(-1)) {
                for (int n = 0; n < 5; n++) { fp[n] = R(0); fm[n] = full[n]; }
            } else if (M >= R(1)) {
                for (int n = 0; n < 5; n++) { fm[n] = R(0); fp[n] = full[n]; }
            } else {
                R unn = un / ss;
                R f1p = rho * c * R(0.25) * sq(M + R(1)) * ss;
                R f1m = -rho * c * R(0.25) * sq(M - R(1)) * ss;
                R t1 = (-unn + R(2) * c) / (g * ss);
                R t2 = (-unn - R(2) * c) / (g * ss);
                R t3 = R(1) / (R(2) * (g * g - R(1)));
                R t4 = R(0.5) * (u * u + v * v + w * w - unn * unn);
                fp[0] = f1p;
                fp[1] = f1p * (A1 * t1 + u);
                fp[2] = f1p * (A2 * t1 + v);
                fp[3] = f1p * (A3 * t1 + w);
                fp[4] = f1p * (sq((g - R(1)) * unn + R(2) * c) * t3 + t4);
                fm[0] = f1m;
                fm[1] = f1m * (A1 * t2 + u);
                fm[2] = f1m * (A2 * t2 + v);
                fm[3] = f1m * (A3 * t2 + w);
                fm[4] = f1m * (sq((g - R(1)) * unn - R(2) * c) * t3 + t4);
            }
        } else {  // split.jl:185-255
            R h = g * p / (rho * (g - R(1))) + R(0.5) * (u * u + v * v + w * w);
            full[0] = rho * un;
            full[1] = rho * u * un + A1 * p;
            full[2] = rho * v * un + A2 * p;
            full[3] = rho * w * un + A3 * p;
            full[4] = rho * h * un;
            if (M <= R(-1)) {
                for (int n = 0; n < 5; n++) { fp[n] = R(0); fm[n] = full[n]; }
            } else if (M >= R(1)) {
                for (int n = 0; n < 5; n++) { fm[n] = R(0); fp[n] = full[n]; }
            } else {
                R f_p = R(0.25) * sq(M + R(1)) * rho * c * ss;
                R f_m = -R(0.25) * sq(M - R(1)) * rho * c * ss;
                R Pp = p * (R(0.25) * sq(M + R(1)) * (R(2) - M));
                R Pm = p * (R(0.25) * sq(M - R(1)) * (R(2) + M));
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
}

// fluxSplit_* over every cell (split.jl), for direction d with metric row A1..A3 and S.
template <class R>
void split(const f3d_params& P, const R* Qp, const R* A1p, const R* A2p, const R* A3p, const R* Sp,
           R* Fpp, R* Fmp) {
    Grid g(P);
    Consts<R> C(P);
    const size_t nc = g.ncell();
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nc; c++) {
        R q[6], fp[5], fm[5];
        for (int n = 0; n < 6; n++) q[n] = Qp[c + n * nc];
        split_cell(P.split_method, C, q, A1p[c], A2p[c], A3p[c], Sp[c], fp, fm);
        for (int n = 0; n < 5; n++) {
            Fpp[c + n * nc] = fp[n];
            Fmp[c + n * nc] = fm[n];
        }
    }
}

// ---------------------------------------------------------------------------------
// Reconstruction building blocks (schemes.jl:119-286 and 813-1009).
// Linear upwind scheme, schemes.jl:129: V1..V7 in the upwind order of the side.
template <class R> inline R linear7(const R* c, const R V[7]) {
    return c[0] * V[0] + c[1] * V[1] + c[2] * V[2] + c[3] * V[3] + c[4] * V[4] + c[5] * V[5] + c[6] * V[6];
}

// WENO7, schemes.jl:153-185. Returns 12x the reconstructed value in the weight type W.
template <class R, class W> inline W weno7(const R V[7], R s0) {
    const R V1 = V[0], V2 = V[1], V3 = V[2], V4 = V[3], V5 = V[4], V6 = V[5], V7 = V[6];
    R q1 = R(-3) * V1 + R(13) * V2 - R(23) * V3 + R(25) * V4;
    R q2 = V2 - R(5) * V3 + R(13) * V4 + R(3) * V5;
    R q3 = -V3 + R(7) * V4 + R(7) * V5 - V6;
    R q4 = R(3) * V4 + R(13) * V5 - R(5) * V6 + V7;
    R Is1 = V1 * (R(547) * V1 - R(3882) * V2 + R(4642) * V3 - R(1854) * V4) +
            V2 * (R(7043) * V2 - R(17246) * V3 + R(7042) * V4) + V3 * (R(11003) * V3 - R(9402) * V4) +
            V4 * (R(2107) * V4);
    R Is2 = V2 * (R(267) * V2 - R(1642) * V3 + R(1602) * V4 - R(494) * V5) +
            V3 * (R(2843) * V3 - R(5966) * V4 + R(1922) * V5) + V4 * (R(3443) * V4 - R(2522) * V5) +
            V5 * (R(547) * V5);
    R Is3 = V3 * (R(547) * V3 - R(2522) * V4 + R(1922) * V5 - R(494) * V6) +
            V4 * (R(3443) * V4 - R(5966) * V5 + R(1602) * V6) + V5 * (R(2843) * V5 - R(1642) * V6) +
            V6 * (R(267) * V6);
    R Is4 = V4 * (R(2107) * V4 - R(9402) * V5 + R(7042) * V6 - R(1854) * V7) +
            V5 * (R(11003) * V5 - R(17246) * V6 + R(4642) * V7) + V6 * (R(7043) * V6 - R(3882) * V7) +
            V7 * (R(547) * V7);
    const W e1 = W(1e-20);
    W a1 = W(1) / sq(e1 + W(Is1 * s0));
    W a2 = W(12) / sq(e1 + W(Is2 * s0));
    W a3 = W(18) / sq(e1 + W(Is3 * s0));
    W a4 = W(4) / sq(e1 + W(Is4 * s0));
    W invsum = W(1) / (a1 + a2 + a3 + a4);
    return invsum * (a1 * W(q1) + a2 * W(q2) + a3 * W(q3) + a4 * W(q4));
}

// WENO5, schemes.jl:233-252. Returns 6x the reconstructed value.
template <class R> inline R weno5(const R V[5], R s0) {
    const R V1 = V[0], V2 = V[1], V3 = V[2], V4 = V[3], V5 = V[4];
    R s11 = R(13) * sq(V1 - R(2) * V2 + V3) + R(3) * sq(V1 - R(4) * V2 + R(3) * V3);
    R s22 = R(13) * sq(V2 - R(2) * V3 + V4) + R(3) * sq(V2 - V4);
    R s33 = R(13) * sq(V3 - R(2) * V4 + V5) + R(3) * sq(R(3) * V3 - R(4) * V4 + V5);
    const R e2 = R(1e-16);
    s11 = R(1) / sq(e2 + s11 * s0);
    s22 = R(6) / sq(e2 + s22 * s0);
    s33 = R(3) / sq(e2 + s33 * s0);
    R invsum = R(1) / (s11 + s22 + s33);
    R v1 = R(2) * V1 - R(7) * V2 + R(11) * V3;
    R v2 = -V2 + R(5) * V3 + R(2) * V4;
    R v3 = R(2) * V3 + R(5) * V4 - V5;
    return invsum * (s11 * v1 + s22 * v2 + s33 * v3);
}

// Branch taken at a face: 0 = UP7 (linear), 1 = WENO7, 2 = WENO5, 3 = NND2.
template <class R> inline int face_branch(const Consts<R>& C, R phimax) {
    if (phimax < C.phi1) return 0;
    if (phimax < C.phi2) return 1;
    if (phimax < C.phi3) return 2;
    return 3;
}

// Face flux of direction d for faces 1..N_d+1 and interior transverse cells; F has the
// shape of Fx/Fy/Fz: (Nx+1,Ny,Nz,5) for d=0 etc. Component-wise = advect_x/y/z
// (schemes.jl:86-698), characteristic = advect_xc/yc/zc (schemes.jl:700-1643). The y
// and z kernels are index permutations of the x kernel. branch_out (optional, F's shape
// without the variable axis) records the branch of every face.
template <class R, class W>
void face_flux(const f3d_params& P, int d, const R* phip, const R* Sp, const R* Fpp, const R* Fmp,
               const R* Qp, const R* A1p, const R* A2p, const R* A3p, R* Fp_out, int8_t* branch_out) {
    Grid g(P);
    Consts<R> C(P);
    const long NG = g.ng;
    const size_t nc = g.ncell();
    const long st = g.stride(d);
    const long fx = g.nx + (d == 0), fy = g.ny + (d == 1), fz = g.nz + (d == 2);
    const size_t nf = (size_t)fx * fy * fz;
    const R tmp1 = R(1) / R(12), tmp2 = R(1) / R(6);
#pragma omp parallel for schedule(static)
    for (long kf = 1; kf <= fz; kf++)
        for (long jf = 1; jf <= fy; jf++)
            for (long ifc = 1; ifc <= fx; ifc++) {
                // cell to the right of the face, 1-based full-grid index
                const long i = ifc + NG, j = jf + NG, k = kf + NG;
                const long c0 = (i - 1) + g.nxt * ((j - 1) + g.nyt * (k - 1));
                auto at = [&](const R* a, long off, int n) -> R { return a[c0 + off * st + (size_t)n * nc]; };
                const size_t fo = (ifc - 1) + fx * ((jf - 1) + fy * (kf - 1));
                R phimax = at(phip, -3, 0);
                for (long o = -2; o <= 2; o++) phimax = jmax(phimax, at(phip, o, 0));
                const int br = face_branch(C, phimax);
                if (branch_out) branch_out[fo] = (int8_t)br;
                R out[5];
                const R s0 = R(2) / (at(Sp, -1, 0) + at(Sp, 0, 0));
                if (br == 0) {  // UP7, schemes.jl:119-142 / 731-754
                    for (int n = 0; n < 5; n++) {
                        R Vp[7], Vm[7];
                        for (int m = 0; m < 7; m++) {
                            Vp[m] = at(Fpp, m - 4, n);
                            Vm[m] = at(Fmp, 3 - m, n);
                        }
                        out[n] = linear7(C.lin, Vp) + linear7(C.lin, Vm);
                    }
                } else if (br == 3) {  // NND2, schemes.jl:277-286 / 1000-1009
                    for (int n = 0; n < 5; n++) {
                        R fp = at(Fpp, -1, n) + R(0.5) * minmod(at(Fpp, 0, n) - at(Fpp, -1, n),
                                                                 at(Fpp, -1, n) - at(Fpp, -2, n));
                        R fm = at(Fmp, 0, n) - R(0.5) * minmod(at(Fmp, 1, n) - at(Fmp, 0, n),
                                                                at(Fmp, 0, n) - at(Fmp, -1, n));
                        out[n] = fp + fm;
                    }
                } else if (!P.character) {  // component-wise WENO7 / WENO5
                    for (int n = 0; n < 5; n++) {
                        if (br == 1) {  // schemes.jl:143-230
                            R Vp[7], Vm[7];
                            for (int m = 0; m < 7; m++) {
                                Vp[m] = at(Fpp, m - 4, n);
                                Vm[m] = at(Fmp, 3 - m, n);
                            }
                            W fp = weno7<R, W>(Vp, s0);
                            W fm = weno7<R, W>(Vm, s0);
                            out[n] = R((fp + fm) * W(tmp1));
                        } else {  // schemes.jl:231-276
                            R Vp[5], Vm[5];
                            for (int m = 0; m < 5; m++) {
                                Vp[m] = at(Fpp, m - 3, n);
                                Vm[m] = at(Fmp, 2 - m, n);
                            }
                            out[n] = (weno5(Vp, s0) + weno5(Vm, s0)) * tmp2;
                        }
                    }
                } else {  // characteristic-wise, schemes.jl:756-999
                    R u = R(0.5) * (at(Qp, 0, 1) + at(Qp, -1, 1));
                    R v = R(0.5) * (at(Qp, 0, 2) + at(Qp, -1, 2));
                    R w = R(0.5) * (at(Qp, 0, 3) + at(Qp, -1, 3));
                    R T = R(0.5) * (at(Qp, 0, 5) + at(Qp, -1, 5));
                    R A1 = (at(A1p, 0, 0) + at(A1p, -1, 0)) * R(0.5);
                    R A2 = (at(A2p, 0, 0) + at(A2p, -1, 0)) * R(0.5);
                    R A3 = (at(A3p, 0, 0) + at(A3p, -1, 0)) * R(0.5);
                    R nx = A1 * s0, ny = A2 * s0, nz = A3 * s0;
                    R lx, ly, lz;
                    if (abs(nz) <= abs(ny)) {
                        R ss = R(1) / sqrt(nx * nx + ny * ny);
                        lx = -ny * ss;
                        ly = nx * ss;
                        lz = R(0);
                    } else {
                        R ss = R(1) / sqrt(nx * nx + nz * nz);
                        lx = -nz * ss;
                        ly = R(0);
                        lz = nx * ss;
                    }
                    R mx = ny * lz - nz * ly;
                    R my = nz * lx - nx * lz;
                    R mz = nx * ly - ny * lx;
                    R qn = u * nx + v * ny + w * nz;
                    R ql = u * lx + v * ly + w * lz;
                    R qm = u * mx + v * my + w * mz;
                    R q2 = R(0.5) * (u * u + v * v + w * w);
                    R c = sqrt(C.gamma * C.rg * T);
                    R c2 = R(1) / (R(2) * c);
                    R K = (C.gamma - R(1)) / (c * c);
                    R K2 = K * R(0.5);
                    R H = R(1) / K + q2;
                    R L[5][5] = {
                        {K2 * q2 + qn * c2, -(K2 * u + nx * c2), -(K2 * v + ny * c2), -(K2 * w + nz * c2), K2},
                        {R(1) - K * q2, K * u, K * v, K * w, -K},
                        {K2 * q2 - qn * c2, -(K2 * u - nx * c2), -(K2 * v - ny * c2), -(K2 * w - nz * c2), K2},
                        {-ql, lx, ly, lz, R(0)},
                        {-qm, mx, my, mz, R(0)}};
                    R Rm[5][5] = {{R(1), R(1), R(1), R(0), R(0)},
                                  {u - c * nx, u, u + c * nx, lx, mx},
                                  {v - c * ny, v, v + c * ny, ly, my},
                                  {w - c * nz, w, w + c * nz, lz, mz},
                                  {H - qn * c, q2, H + qn * c, ql, qm}};
                    R flux[5];
                    const int np = br == 1 ? 7 : 5;
                    const int lo = br == 1 ? -4 : -3;  // first Fp point
                    const int hi = br == 1 ? 3 : 2;    // first Fm point
                    for (int n = 0; n < 5; n++) {
                        R Fpc[7], Fmc[7];
                        for (int m = 0; m < np; m++) { Fpc[m] = R(0); Fmc[m] = R(0); }
                        for (int m = 0; m < 5; m++) {
                            const R ll = L[n][m];
                            for (int s = 0; s < np; s++) {
                                Fpc[s] += at(Fpp, lo + s, m) * ll;
                                Fmc[s] += at(Fmp, hi - s, m) * ll;
                            }
                        }
                        if (br == 1) {
                            W fp = weno7<R, W>(Fpc, s0);
                            W fm = weno7<R, W>(Fmc, s0);
                            flux[n] = R((fp + fm) * W(tmp1));
                        } else {
                            flux[n] = (weno5(Fpc, s0) + weno5(Fmc, s0)) * tmp2;
                        }
                    }
                    for (int n = 0; n < 5; n++)
                        out[n] = flux[0] * Rm[n][0] + flux[1] * Rm[n][1] + flux[2] * Rm[n][2] +
                                 flux[3] * Rm[n][3] + flux[4] * Rm[n][4];
                }
                for (int n = 0; n < 5; n++) Fp_out[fo + n * nf] = out[n];
            }
}

// ---------------------------------------------------------------------------------
// viscous.jl:1-64, 107-133 viscousFlux (laminar; the LES branches are off by default).
// Fv arrays are (Nt-4)^3 x 4 with Fv index = cell index - 2.
template <class R>
void viscous(const f3d_params& P, const R* Qp, const R* const m[9], const R* Jp, R* Fvxp, R* Fvyp, R* Fvzp) {
    Grid g(P);
    Consts<R> C(P);
    V4<const R> Q{Qp, g.nxt, g.nyt, g.nzt};
    const long vx = g.nxt - 4, vy = g.nyt - 4, vz = g.nzt - 4;
    V4<R> Fvx{Fvxp, vx, vy, vz}, Fvy{Fvyp, vx, vy, vz}, Fvz{Fvzp, vx, vy, vz};
    const R c1 = R(1) / R(12), c2 = R(-2) / R(3), c23 = R(2) / R(3);
#pragma omp parallel for schedule(static)
    for (long k = 3; k <= g.nzt - 2; k++)
        for (long j = 3; j <= g.nyt - 2; j++)
            for (long i = 3; i <= g.nxt - 2; i++) {
                const size_t c = (i - 1) + g.nxt * ((j - 1) + g.nyt * (k - 1));
                R xx = m[0][c], xy = m[1][c], xz = m[2][c];
                R ex = m[3][c], ey = m[4][c], ez = m[5][c];
                R zx = m[6][c], zy = m[7][c], zz = m[8][c];
                R Jac = Jp[c];
                R T = Q(i, j, k, 6);
                R mu = C.c_s * T * sqrt(T) / (T + C.t_s);
                R lam = C.cp * mu / C.pr;
                auto dxi = [&](int n) { return c1 * (Q(i - 2, j, k, n) - Q(i + 2, j, k, n)) + c2 * (Q(i - 1, j, k, n) - Q(i + 1, j, k, n)); };
                auto deta = [&](int n) { return c1 * (Q(i, j - 2, k, n) - Q(i, j + 2, k, n)) + c2 * (Q(i, j - 1, k, n) - Q(i, j + 1, k, n)); };
                auto dzeta = [&](int n) { return c1 * (Q(i, j, k - 2, n) - Q(i, j, k + 2, n)) + c2 * (Q(i, j, k - 1, n) - Q(i, j, k + 1, n)); };
                R uxi = dxi(2), vxi = dxi(3), wxi = dxi(4), Txi = dxi(6);
                R ueta = deta(2), veta = deta(3), weta = deta(4), Teta = deta(6);
                R uze = dzeta(2), vze = dzeta(3), wze = dzeta(4), Tze = dzeta(6);
                R u = Q(i, j, k, 2), v = Q(i, j, k, 3), w = Q(i, j, k, 4);
                R dudx = (uxi * xx + ueta * ex + uze * zx) * Jac;
                R dudy = (uxi * xy + ueta * ey + uze * zy) * Jac;
                R dudz = (uxi * xz + ueta * ez + uze * zz) * Jac;
                R dvdx = (vxi * xx + veta * ex + vze * zx) * Jac;
                R dvdy = (vxi * xy + veta * ey + vze * zy) * Jac;
                R dvdz = (vxi * xz + veta * ez + vze * zz) * Jac;
                R dwdx = (wxi * xx + weta * ex + wze * zx) * Jac;
                R dwdy = (wxi * xy + weta * ey + wze * zy) * Jac;
                R dwdz = (wxi * xz + weta * ez + wze * zz) * Jac;
                R dTdx = (Txi * xx + Teta * ex + Tze * zx) * Jac;
                R dTdy = (Txi * xy + Teta * ey + Tze * zy) * Jac;
                R dTdz = (Txi * xz + Teta * ez + Tze * zz) * Jac;
                R dv = dudx + dvdy + dwdz;
                if (P.les) {  // viscous.jl:66-106, Pr_t = 0.9
                    const R rho = Q(i, j, k, 1);
                    const R s12 = R(0.5) * (dudy + dvdx), s13 = R(0.5) * (dudz + dwdx), s23 = R(0.5) * (dvdz + dwdy);
                    const R sii = dudx * dudx + dvdy * dvdy + dwdz * dwdz;
                    const R sij = s12 * s12 + s13 * s13 + s23 * s23;
                    // Jac^(1/3f0), S^5 and Sd^2.5f0 through pow, (C/Jac^(1/3))^2 and Sd^3 as
                    // Julia's literal powers (products), in the reference's grouping
                    const R J13 = pow(Jac, R(1) / R(3));
                    R mut;
                    if (P.les == F3D_LES_SMAGORINSKY) {  // viscous.jl:66-78
                        const R Smag = sqrt(R(2) * (sii + R(2) * sij));
                        const R cd = R(0.1) / J13;
                        mut = jmin(rho * (cd * cd) * Smag, R(2) * mu);
                    } else {  // WALE, viscous.jl:79-101
                        const R S = sqrt(sii + R(2) * sij);
                        R d11 = dudx * dudx + dudy * dvdx + dudz * dwdx;
                        R d22 = dvdx * dudy + dvdy * dvdy + dvdz * dwdy;
                        R d33 = dwdx * dudz + dwdy * dvdz + dwdz * dwdz;
                        const R tr = R(1) / R(3) * (d11 + d22 + d33);
                        d11 = d11 - tr;
                        d22 = d22 - tr;
                        d33 = d33 - tr;
                        const R d12 = R(0.5) * (dudx * dvdx + dvdx * dvdy + dwdx * dvdz + dudy * dudx + dvdy * dudy + dwdy * dudz);
                        const R d13 = R(0.5) * (dudx * dwdx + dvdx * dwdy + dwdx * dwdz + dudz * dudx + dvdz * dudy + dwdz * dudz);
                        const R d23 = R(0.5) * (dudy * dwdx + dvdy * dwdy + dwdy * dwdz + dudz * dvdx + dvdz * dvdy + dwdz * dvdz);
                        const R Sd = sqrt(d11 * d11 + d22 * d22 + d33 * d33 + R(2) * (d12 * d12 + d13 * d13 + d23 * d23));
                        const R D = Sd * Sd * Sd / (pow(S, R(5)) + pow(Sd, R(2.5)));  // Sd^3/(S^5 + Sd^2.5)
                        const R cd = R(0.325) / J13;
                        mut = jmin(rho * (cd * cd) * D, R(2) * mu);
                    }
                    mu = mu + mut;
                    lam = lam + C.cp * mut / R(0.9);
                }
                R t11 = mu * (R(2) * dudx - c23 * dv);
                R t12 = mu * (dudy + dvdx);
                R t13 = mu * (dudz + dwdx);
                R t22 = mu * (R(2) * dvdy - c23 * dv);
                R t23 = mu * (dwdy + dvdz);
                R t33 = mu * (R(2) * dwdz - c23 * dv);
                R E1 = u * t11 + v * t12 + w * t13 + lam * dTdx;
                R E2 = u * t12 + v * t22 + w * t23 + lam * dTdy;
                R E3 = u * t13 + v * t23 + w * t33 + lam * dTdz;
                const long a = i - 2, b = j - 2, e = k - 2;
                Fvx(a, b, e, 1) = xx * t11 + xy * t12 + xz * t13;
                Fvx(a, b, e, 2) = xx * t12 + xy * t22 + xz * t23;
                Fvx(a, b, e, 3) = xx * t13 + xy * t23 + xz * t33;
                Fvx(a, b, e, 4) = xx * E1 + xy * E2 + xz * E3;
                Fvy(a, b, e, 1) = ex * t11 + ey * t12 + ez * t13;
                Fvy(a, b, e, 2) = ex * t12 + ey * t22 + ez * t23;
                Fvy(a, b, e, 3) = ex * t13 + ey * t23 + ez * t33;
                Fvy(a, b, e, 4) = ex * E1 + ey * E2 + ez * E3;
                Fvz(a, b, e, 1) = zx * t11 + zy * t12 + zz * t13;
                Fvz(a, b, e, 2) = zx * t12 + zy * t22 + zz * t23;
                Fvz(a, b, e, 3) = zx * t13 + zy * t23 + zz * t33;
                Fvz(a, b, e, 4) = zx * E1 + zy * E2 + zz * E3;
            }
}

// ---------------------------------------------------------------------------------
// div.jl:1-50. With U_inout != null: U += (dF)*Jact, then U[2..5] += (dFv)*Jact with
// Jact = J*dt (the reference's fused Euler update). With dUdt != null: dUdt = dF*J + dFv*J
// (the right-hand side itself, the same two-term structure without dt).
template <class R>
void divergence(const f3d_params& P, const R* Fxp, const R* Fyp, const R* Fzp, const R* Fvxp,
                const R* Fvyp, const R* Fvzp, const R* Jp, R dt, R* U_inout, R* dUdt, const R* dtl = nullptr) {
    Grid g(P);
    const long NG = g.ng;
    const long Nx = g.nx, Ny = g.ny, Nz = g.nz;
    V4<const R> Fx{Fxp, Nx + 1, Ny, Nz}, Fy{Fyp, Nx, Ny + 1, Nz}, Fz{Fzp, Nx, Ny, Nz + 1};
    const long vx = g.nxt - 4, vy = g.nyt - 4, vz = g.nzt - 4;
    V4<const R> Fvx{Fvxp, vx, vy, vz}, Fvy{Fvyp, vx, vy, vz}, Fvz{Fvzp, vx, vy, vz};
    V4<const R> Jv{Jp, g.nxt, g.nyt, g.nzt};
    V4<R> U{U_inout, g.nxt, g.nyt, g.nzt}, D{dUdt, g.nxt, g.nyt, g.nzt};
    const R c1 = R(1) / R(12), c2 = R(-2) / R(3);
    const bool visc = Fvxp != nullptr;
#pragma omp parallel for schedule(static)
    for (long k = 1; k <= Nz; k++)
        for (long j = 1; j <= Ny; j++)
            for (long i = 1; i <= Nx; i++) {
                const R Jc = Jv(i + NG, j + NG, k + NG);
                // div_LTS (div.jl:52-101) with a per-cell dt
                const R dtc = dtl ? dtl[(i + NG - 1) + g.nxt * ((j + NG - 1) + g.nyt * (k + NG - 1))] : dt;
                const R Jact = U_inout ? Jc * dtc : Jc;
                R dv[5] = {R(0), R(0), R(0), R(0), R(0)};
                if (visc) {
                    for (int n = 1; n <= 4; n++) {
                        R a = c1 * (Fvx(i, j + 2, k + 2, n) - Fvx(i + 4, j + 2, k + 2, n)) +
                              c2 * (Fvx(i + 1, j + 2, k + 2, n) - Fvx(i + 3, j + 2, k + 2, n));
                        R b = c1 * (Fvy(i + 2, j, k + 2, n) - Fvy(i + 2, j + 4, k + 2, n)) +
                              c2 * (Fvy(i + 2, j + 1, k + 2, n) - Fvy(i + 2, j + 3, k + 2, n));
                        R e = c1 * (Fvz(i + 2, j + 2, k, n) - Fvz(i + 2, j + 2, k + 4, n)) +
                              c2 * (Fvz(i + 2, j + 2, k + 1, n) - Fvz(i + 2, j + 2, k + 3, n));
                        dv[n] = a + b + e;
                    }
                }
                for (int n = 1; n <= 5; n++) {
                    R inv = Fx(i, j, k, n) - Fx(i + 1, j, k, n) + Fy(i, j, k, n) - Fy(i, j + 1, k, n) +
                            Fz(i, j, k, n) - Fz(i, j, k + 1, n);
                    if (U_inout) {
                        R& u = U(i + NG, j + NG, k + NG, n);
                        u += inv * Jact;
                        if (visc && n >= 2) u += dv[n - 1] * Jact;
                    } else {
                        R r = inv * Jact;
                        if (visc && n >= 2) r += dv[n - 1] * Jact;
                        D(i + NG, j + NG, k + NG, n) = r;
                    }
                }
            }
}

// |grad xi_d| at every cell, solver.jl:286-288.
template <class R> void metric_norm(size_t nc, const R* a, const R* b, const R* c, R* s) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)nc; i++) s[i] = sqrt(a[i] * a[i] + b[i] * b[i] + c[i] * c[i]);
}

// utils.jl:73-99 compute_dt: interior cells, LTS_CFL * min(V/S1/(u+c), V/S2/(v+c), V/S3/(w+c)).
template <class R>
void compute_dt(const f3d_params& P, const R* Qp, const R* Jp, const R* S1, const R* S2, const R* S3, R* dtp) {
    Grid g(P);
    Consts<R> C(P);
    V4<const R> Q{Qp, g.nxt, g.nyt, g.nzt};
    const R cfl = R(P.lts_cfl);
#pragma omp parallel for schedule(static)
    for (long k = g.ng + 1; k <= g.nz + g.ng; k++)
        for (long j = g.ng + 1; j <= g.ny + g.ng; j++)
            for (long i = g.ng + 1; i <= g.nx + g.ng; i++) {
                const size_t c = Q.lin(i, j, k);
                const R u = Q(i, j, k, 2), v = Q(i, j, k, 3), w = Q(i, j, k, 4), T = Q(i, j, k, 6);
                const R V = R(1) / Jp[c];
                const R cs = sqrt(C.gamma * C.rg * T);
                const R dtx = V / S1[c] / (u + cs), dty = V / S2[c] / (v + cs), dtz = V / S3[c] / (w + cs);
                dtp[c] = jmin(jmin(dtx, dty), dtz) * cfl;
            }
}

// The explicit filters of one direction d over interior cells (utils.jl:102-315): the
// shock-capturing pair pre_x/filter_x (nonlinear) or linearFilter_x, from Un into U.
template <class R>
void filter_dir(const f3d_params& P, int d, const R* Qp, R* Up, const R* Unp, R* scp) {
    Grid g(P);
    const long NG = g.ng, st = g.stride(d);
    const size_t nc = g.ncell();
    const R s0 = R(P.filter_s0), rth = R(P.filter_rth);
    auto interior = [&](auto&& fn) {
#pragma omp parallel for schedule(static)
        for (long k = NG + 1; k <= g.nz + NG; k++)
            for (long j = NG + 1; j <= g.ny + NG; j++)
                for (long i = NG + 1; i <= g.nx + NG; i++) fn((size_t)((i - 1) + g.nxt * ((j - 1) + g.nyt * (k - 1))));
    };
    if (P.filter == F3D_FILTER_NONLINEAR) {
        interior([&](size_t c) {  // pre_x, utils.jl:102-123
            const R* p = Qp + 4 * nc + c;
            const R p1 = p[-2 * st], p2 = p[-st], p3 = p[0], p4 = p[st], p5 = p[2 * st];
            const R d0 = R(0.25) * (-p4 + R(2) * p3 - p2);
            const R d1 = R(0.25) * (-p5 + R(2) * p4 - p3);
            const R d2 = R(0.25) * (-p3 + R(2) * p2 - p1);
            const R ri = R(0.5) * ((d0 - d1) * (d0 - d1) + (d0 - d2) * (d0 - d2)) / (p3 * p3) + R(1e-16);
            scp[c] = R(0.5) * (R(1) - rth / ri + abs(R(1) - rth / ri));
        });
        interior([&](size_t c) {  // filter_x, utils.jl:171-193
            const R c1 = R(-0.210383), c2 = R(0.039617);
            const R sc1 = R(0.5) * (scp[c] + scp[c + st]), sc2 = R(0.5) * (scp[c] + scp[c - st]);
            for (int n = 0; n < 5; n++) {
                const R* f = Unp + n * nc + c;
                Up[n * nc + c] = f[0] - s0 * (sc1 * (c1 * (f[st] - f[0]) + c2 * (f[2 * st] - f[-st])) -
                                              sc2 * (c1 * (f[0] - f[-st]) + c2 * (f[st] - f[-2 * st])));
            }
        });
    } else {
        interior([&](size_t c) {  // linearFilter_x, utils.jl:243-266
            const R d0 = R(0.243527493120), d1 = R(-0.204788880640), d2 = R(0.120007591680),
                    d3 = R(-0.045211119360), d4 = R(0.008228661760);
            for (int n = 0; n < 5; n++) {
                const R* f = Unp + n * nc + c;
                Up[n * nc + c] = f[0] - s0 * (d0 * f[0] + d1 * (f[-st] + f[st]) + d2 * (f[-2 * st] + f[2 * st]) +
                                              d3 * (f[-3 * st] + f[3 * st]) + d4 * (f[-4 * st] + f[4 * st]));
            }
        });
    }
}

}  // namespace f3do
#include "f3d_oracle_fvm.hpp"
namespace f3do {

// ---------------------------------------------------------------------------------
// Workspace and the composed RHS / RK3 stage (solver.jl:416-444 with flowAdvance).
// The finite-volume schemes (params.scheme) reconstruct U: the stage's state, or prim2c(Q)
// for a bare RHS; they need the cell-centre coordinates (set_coordinates). Their face geometry
// is computed in G: R, except for long double, whose solver (the rounding yardstick) takes
// the FP64 geometry and so the FP64 side of every |nz| = |ny| tie of the tangent basis.
template <class R, class W> struct Solver {
    using G = typename std::conditional<std::is_same<R, long double>::value, double, R>::type;
    f3d_params P;
    Grid g;
    const R* m[9];
    const R* J;
    const G *xs = nullptr, *ys = nullptr, *zs = nullptr;
    std::vector<R> S[3], phi, Fp, Fm, F[3], Fv[3], Uq, dtl, sc;
    std::vector<G> xyz[3];
    long tt = 0;  // steps done (the filter runs after every filter_interval-th)
    std::vector<int8_t> branch[3];
    bool record_branch = false;

    Solver(const f3d_params& p, const R* const metrics[9], const R* jac) : P(p), g(p) {
        for (int i = 0; i < 9; i++) m[i] = metrics[i];
        J = jac;
        const size_t nc = g.ncell();
        for (int d = 0; d < 3; d++) {
            S[d].assign(nc, R(0));
            metric_norm(nc, m[3 * d], m[3 * d + 1], m[3 * d + 2], S[d].data());
            const size_t nf = (size_t)(g.nx + (d == 0)) * (g.ny + (d == 1)) * (g.nz + (d == 2));
            F[d].assign(nf * 5, R(0));
            Fv[d].assign((size_t)(g.nxt - 4) * (g.nyt - 4) * (g.nzt - 4) * 4, R(0));
            branch[d].assign(nf, 0);
        }
        phi.assign(nc, R(0));  // CUDA.zeros: cells 1 and Nt are never written
        if (P.scheme != F3D_SCHEME_FDM && coordinates()[0]) {
            for (int a = 0; a < 3; a++) xyz[a].assign(coordinates()[a], coordinates()[a] + nc);
            set_coordinates(xyz[0].data(), xyz[1].data(), xyz[2].data());
        }
        Fp.assign(nc * 5, R(0));
        Fm.assign(nc * 5, R(0));
    }

    void set_coordinates(const G* x, const G* y, const G* z) {
        xs = x;
        ys = y;
        zs = z;
    }

    // shockSensor + the flux part of flowAdvance: fills F[0..2] and Fv[0..2].
    void fluxes(const R* Q, const R* U = nullptr) {
        sensor<R>(P, Q, phi.data());
        if (P.scheme != F3D_SCHEME_FDM) {  // FVM.jl (solver.jl:21-31)
            if (!U) {
                Uq.assign(g.ncell() * 5, R(0));
                prim2c<R>(P, Q, Uq.data());
                U = Uq.data();
            }
            for (int d = 0; d < 3; d++)
                fvm_face_flux<R, G>(P, d, P.scheme == F3D_SCHEME_FVM_EIGEN, phi.data(), S[d].data(), Q, U, xs, ys, zs,
                                 F[d].data(), record_branch ? branch[d].data() : nullptr);
            if (P.viscous) viscous<R>(P, Q, m, J, Fv[0].data(), Fv[1].data(), Fv[2].data());
            return;
        }
        for (int d = 0; d < 3; d++) {
            split<R>(P, Q, m[3 * d], m[3 * d + 1], m[3 * d + 2], S[d].data(), Fp.data(), Fm.data());
            face_flux<R, W>(P, d, phi.data(), S[d].data(), Fp.data(), Fm.data(), Q, m[3 * d], m[3 * d + 1],
                            m[3 * d + 2], F[d].data(), record_branch ? branch[d].data() : nullptr);
        }
        if (P.viscous) viscous<R>(P, Q, m, J, Fv[0].data(), Fv[1].data(), Fv[2].data());
    }

    void rhs(const R* Q, R* dUdt) {
        fluxes(Q);
        const bool v = P.viscous != 0;
        divergence<R>(P, F[0].data(), F[1].data(), F[2].data(), v ? Fv[0].data() : nullptr,
                      v ? Fv[1].data() : nullptr, v ? Fv[2].data() : nullptr, J, R(0), nullptr, dUdt);
    }

    // solver.jl:416-444, one stage.
    void rk3_stage(int stage, R dt, R* U, R* Un, R* Q) {
        const size_t n5 = g.ncell() * 5;
        if (stage == 1) std::memcpy(Un, U, n5 * sizeof(R));
        // solver.jl:418-421: compute_dt inside `if KRK == 1`, before flowAdvance; stages 2
        // and 3 take the first stage's steps (a lone later stage on a fresh solver computes
        // them from its own Q, having no first stage)
        if (P.lts && (stage == 1 || dtl.empty())) {
            dtl.assign(g.ncell(), R(0));
            compute_dt<R>(P, Q, J, S[0].data(), S[1].data(), S[2].data(), dtl.data());
        }
        fluxes(Q, U);
        const bool v = P.viscous != 0;
        divergence<R>(P, F[0].data(), F[1].data(), F[2].data(), v ? Fv[0].data() : nullptr,
                      v ? Fv[1].data() : nullptr, v ? Fv[2].data() : nullptr, J, dt, U, nullptr,
                      P.lts ? dtl.data() : nullptr);
        if (stage == 2) lincomb<R>(P, U, Un, R(0.25), R(0.75));
        if (stage == 3) lincomb<R>(P, U, Un, R(2) / R(3), R(1) / R(3));
        c2prim<R>(P, U, Q);
        fill_ghosts<R>(P, Q, U);
    }

    // solver.jl:446-470 after a step: the filter every filter_interval steps, each
    // direction from a copy Un of U (Q unchanged).
    void after_step(R* U, R* Un, const R* Q) {
        tt++;
        if (!P.filter || tt % P.filter_interval != 0) return;
        if (sc.empty()) sc.assign(g.ncell(), R(0));
        for (int d = 0; d < 3; d++) {
            std::memcpy(Un, U, g.ncell() * 5 * sizeof(R));
            filter_dir<R>(P, d, Q, U, Un, sc.data());
        }
    }

    void rk3_step(R dt, R* U, R* Un, R* Q) {
        for (int st = 1; st <= 3; st++) rk3_stage(st, dt, U, Un, Q);
        after_step(U, Un, Q);
    }
};

// ---------------------------------------------------------------------------------
// parse_mesh.jl:139-248: CD6 in the interior, one-sided CD2 in the three outer layers,
// J = 1/det, metrics = cofactors (J^-1-scaled, parse_mesh.jl:239).
template <class R>
void metrics_from_coords(const f3d_params& P, const R* x, const R* y, const R* z, R* const m[9], R* Jout) {
    Grid g(P);
    const size_t nc = g.ncell();
    std::vector<R> d[9];  // dx/dxi, dy/dxi, dz/dxi, dx/deta, ..., dz/dzeta
    for (auto& a : d) a.assign(nc, R(0));
    const R* X[3] = {x, y, z};
    for (int dir = 0; dir < 3; dir++) {
        const long Nt = g.nt(dir), st = g.stride(dir);
#pragma omp parallel for schedule(static)
        for (long c = 0; c < (long)nc; c++) {
            long idx[3] = {c % g.nxt, (c / g.nxt) % g.nyt, c / (g.nxt * g.nyt)};
            long ii = idx[dir] + 1;  // 1-based index along dir
            for (int comp = 0; comp < 3; comp++) {
                const R* f = X[comp] + c;
                R val;
                if (ii >= 4 && ii <= Nt - 3) {
                    val = R(1.0 / 60) * (f[3 * st] - f[-3 * st]) - R(3.0 / 20) * (f[2 * st] - f[-2 * st]) +
                          R(3.0 / 4) * (f[st] - f[-st]);
                } else if (ii <= 3) {
                    val = R(2) * f[st] - R(0.5) * f[2 * st] - R(1.5) * f[0];
                } else {
                    val = R(-2) * f[-st] + R(0.5) * f[-2 * st] + R(1.5) * f[0];
                }
                d[3 * dir + comp][c] = val;
            }
        }
    }
    const R *xxi = d[0].data(), *yxi = d[1].data(), *zxi = d[2].data();
    const R *xet = d[3].data(), *yet = d[4].data(), *zet = d[5].data();
    const R *xze = d[6].data(), *yze = d[7].data(), *zze = d[8].data();
#pragma omp parallel for schedule(static)
    for (long c = 0; c < (long)nc; c++) {
        Jout[c] = R(1) / (xxi[c] * (yet[c] * zze[c] - yze[c] * zet[c]) - xet[c] * (yxi[c] * zze[c] - yze[c] * zxi[c]) +
                          xze[c] * (yxi[c] * zet[c] - yet[c] * zxi[c]));
        m[0][c] = yet[c] * zze[c] - yze[c] * zet[c];
        m[1][c] = xze[c] * zet[c] - xet[c] * zze[c];
        m[2][c] = xet[c] * yze[c] - xze[c] * yet[c];
        m[3][c] = yze[c] * zxi[c] - yxi[c] * zze[c];
        m[4][c] = xxi[c] * zze[c] - xze[c] * zxi[c];
        m[5][c] = xze[c] * yxi[c] - xxi[c] * yze[c];
        m[6][c] = yxi[c] * zet[c] - yet[c] * zxi[c];
        m[7][c] = xet[c] * zxi[c] - xxi[c] * zet[c];
        m[8][c] = xxi[c] * yet[c] - xet[c] * yxi[c];
    }
}

}  // namespace f3do
