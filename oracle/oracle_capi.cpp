// oracle_capi.cpp — extern "C" entry points of the CPU oracle (liboracle_f3d.so).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline through ctypes. All arrays are host arrays in the reference layout.
// orc_* work in FP64; orc32_* mirror the reference's Float32 arithmetic (WENO7 alphas in
// Float64). The JVP entry points run the same templates on dual numbers.
#include <omp.h>

#include <cstring>
#include <vector>

#include "f3d_numtypes.hpp"
#include "f3d_oracle.hpp"

using namespace f3do;

extern "C" {

int orc_set_threads(int n) {
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
}

// compute_dt (utils.jl:73-99) into dt at interior cells; one filter pass (3 directions).
void orc_local_dt(const f3d_params* P, const double* Q, const double* const m[9], const double* J, double* dt) {
    Solver<double, double> s(*P, m, J);
    compute_dt<double>(*P, Q, J, s.S[0].data(), s.S[1].data(), s.S[2].data(), dt);
}
void orc_filter(const f3d_params* P, double* U, double* Un, const double* Q) {
    Grid g(*P);
    std::vector<double> sc(g.ncell(), 0.0);
    for (int d = 0; d < 3; d++) {
        std::memcpy(Un, U, g.ncell() * 5 * sizeof(double));
        filter_dir<double>(*P, d, Q, U, Un, sc.data());
    }
}

// Register (or clear, with nullptrs) the cell-centre coordinates the finite-volume schemes
// take their face geometry from.
void orc_set_coordinates(const double* x, const double* y, const double* z) {
    coordinates()[0] = x;
    coordinates()[1] = y;
    coordinates()[2] = z;
}

// FVM.jl face fluxes of direction dir (Fx/Fy/Fz shape) from ghost-filled Q and U.
void orc_fvm_face_flux(const f3d_params* P, int dir, int eigen, const double* phi, const double* S, const double* Q,
                       const double* U, const double* x, const double* y, const double* z, double* F,
                       int8_t* branch) {
    fvm_face_flux<double>(*P, dir, eigen != 0, phi, S, Q, U, x, y, z, F, branch);
}

// Register (or clear, with nullptr) the state array of an inflow-profile face.
void orc_set_inflow_profile(int face, const double* prof) {
    if (face >= 0 && face < 6) inflow_profile(face) = prof;
}

// Register (or clear) the tangent of an inflow profile for the dual-number entries.
void orc_set_inflow_profile_tangent(int face, const double* dprof) {
    if (face >= 0 && face < 6) inflow_profile_tangent(face) = dprof;
}

void orc_c2prim(const f3d_params* P, const double* U, double* Q) { c2prim<double>(*P, U, Q); }
void orc_prim2c(const f3d_params* P, const double* Q, double* U) { prim2c<double>(*P, Q, U); }
void orc_lincomb(const f3d_params* P, double* U, const double* Un, double a, double b) {
    lincomb<double>(*P, U, Un, a, b);
}
void orc_fill_ghosts(const f3d_params* P, double* Q, double* U) { fill_ghosts<double>(*P, Q, U); }
void orc_sensor(const f3d_params* P, const double* Q, double* phi) { sensor<double>(*P, Q, phi); }
void orc_metric_norm(const f3d_params* P, const double* a, const double* b, const double* c, double* s) {
    metric_norm<double>(Grid(*P).ncell(), a, b, c, s);
}
void orc_split(const f3d_params* P, const double* Q, const double* A1, const double* A2, const double* A3,
               const double* S, double* Fp, double* Fm) {
    split<double>(*P, Q, A1, A2, A3, S, Fp, Fm);
}
void orc_face_flux(const f3d_params* P, int dir, const double* phi, const double* S, const double* Fp,
                   const double* Fm, const double* Q, const double* A1, const double* A2, const double* A3,
                   double* F, int8_t* branch) {
    face_flux<double, double>(*P, dir, phi, S, Fp, Fm, Q, A1, A2, A3, F, branch);
}
void orc_viscous(const f3d_params* P, const double* Q, const double* const m[9], const double* J, double* Fvx,
                 double* Fvy, double* Fvz) {
    viscous<double>(*P, Q, m, J, Fvx, Fvy, Fvz);
}
void orc_divergence(const f3d_params* P, const double* Fx, const double* Fy, const double* Fz, const double* Fvx,
                    const double* Fvy, const double* Fvz, const double* J, double dt, double* U_inout,
                    double* dUdt) {
    divergence<double>(*P, Fx, Fy, Fz, Fvx, Fvy, Fvz, J, dt, U_inout, dUdt);
}
void orc_metrics(const f3d_params* P, const double* x, const double* y, const double* z, double* const m[9],
                 double* J) {
    metrics_from_coords<double>(*P, x, y, z, m, J);
}

// Full RHS from a ghost-filled Q. branches (optional) receives the branch map of the
// three directions concatenated (Fx, Fy, Fz face shapes).
void orc_rhs(const f3d_params* P, const double* Q, const double* const m[9], const double* J, double* dUdt,
             int8_t* branches) {
    Solver<double, double> s(*P, m, J);
    s.record_branch = branches != nullptr;
    s.rhs(Q, dUdt);
    if (branches) {
        size_t off = 0;
        for (int d = 0; d < 3; d++) {
            std::memcpy(branches + off, s.branch[d].data(), s.branch[d].size());
            off += s.branch[d].size();
        }
    }
}

// nsteps SSP-RK3 steps (solver.jl:410-444). U, Un, Q updated in place.
void orc_rk3(const f3d_params* P, int nsteps, double dt, double* U, double* Un, double* Q,
             const double* const m[9], const double* J) {
    Solver<double, double> s(*P, m, J);
    for (int t = 0; t < nsteps; t++)
        s.rk3_step(dt, U, Un, Q);
}

// Persistent workspace for timing: create once, step many times (allocation is set-up
// work in the reference too, solver.jl:293-337).
void* orc_solver_create(const f3d_params* P, const double* const m[9], const double* J) {
    return new Solver<double, double>(*P, m, J);
}
void orc_solver_rk3(void* h, int nsteps, double dt, double* U, double* Un, double* Q) {
    auto* s = static_cast<Solver<double, double>*>(h);
    for (int t = 0; t < nsteps; t++)
        s->rk3_step(dt, U, Un, Q);
}
void orc_solver_destroy(void* h) { delete static_cast<Solver<double, double>*>(h); }

// One stage (for stage-by-stage parity).
void orc_rk3_stage(const f3d_params* P, int stage, double dt, double* U, double* Un, double* Q,
                   const double* const m[9], const double* J) {
    Solver<double, double> s(*P, m, J);
    s.rk3_stage(stage, dt, U, Un, Q);
}

// ---- extended precision (long double: 80-bit on x86-64, 128-bit on aarch64) ------------
// The same formulas with a longer significand: the yardstick for the rounding error of
// any FP64 evaluation (the FP64 oracle's own and the GPU's).
void orcld_rhs(const f3d_params* P, const double* Q, const double* const m[9], const double* J, double* dUdt,
               double* flux_scale) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using L = long double;
    std::vector<L> Ql(Q, Q + nc * 6), R(nc * 5, L(0)), ml[9], Jl(J, J + nc);
    const L* mp[9];
    for (int a = 0; a < 9; a++) {
        ml[a].assign(m[a], m[a] + nc);
        mp[a] = ml[a].data();
    }
    Solver<L, L> s(*P, mp, Jl.data());
    s.rhs(Ql.data(), R.data());
    for (size_t i = 0; i < nc * 5; i++) dUdt[i] = (double)R[i];
    if (flux_scale) {
        // per variable: max over interior cells of J * sum over directions of |F_left| + |F_right|
        // (+ the four viscous terms), the magnitude of what the RHS differences.
        const long NG = g.ng;
        for (int n = 0; n < 5; n++) flux_scale[n] = 0.0;
        for (long k = 0; k < g.nz; k++)
            for (long j = 0; j < g.ny; j++)
                for (long i = 0; i < g.nx; i++) {
                    const size_t c = (i + NG) + g.nxt * ((j + NG) + g.nyt * (k + NG));
                    for (int n = 0; n < 5; n++) {
                        long double acc = 0;
                        for (int d = 0; d < 3; d++) {
                            const long fx = g.nx + (d == 0), fy = g.ny + (d == 1);
                            const size_t nf = (size_t)fx * fy * (g.nz + (d == 2));
                            const size_t f0 = i + fx * (j + fy * k);
                            const size_t f1 = f0 + (d == 0 ? 1 : (d == 1 ? fx : (size_t)fx * fy));
                            acc += fabsl(s.F[d][f0 + n * nf]) + fabsl(s.F[d][f1 + n * nf]);
                        }
                        double v = (double)(fabsl(Jl[c]) * acc);
                        if (v > flux_scale[n]) flux_scale[n] = v;
                    }
                }
    }
}

// Finite-volume face fluxes of one direction in long double from FP64 inputs (rounded back),
// on the FP64 face geometry.
void orcld_fvm_face_flux(const f3d_params* P, int dir, int eigen, const double* phi, const double* S,
                         const double* Q, const double* U, const double* x, const double* y, const double* z,
                         double* F) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using L = long double;
    std::vector<L> phil(phi, phi + nc), Sl(S, S + nc), Ql(Q, Q + nc * 6), Ul(U, U + nc * 5);
    const size_t nf = (size_t)(g.nx + (dir == 0)) * (g.ny + (dir == 1)) * (g.nz + (dir == 2));
    std::vector<L> Fl(nf * 5, L(0));
    // the face geometry in FP64 (the FP64 normals), the rest in long double
    fvm_face_flux<L, double>(*P, dir, eigen != 0, phil.data(), Sl.data(), Ql.data(), Ul.data(), x, y, z, Fl.data(),
                             nullptr);
    for (size_t i = 0; i < nf * 5; i++) F[i] = (double)Fl[i];
}

// ---- the reference's own precision: Float32 state, Float64 WENO7 alphas -------------
// nsteps SSP-RK3 steps in long double from FP64 inputs (the yardstick for the rounding of
// FP64 trajectories); U, Un, Q updated in place (rounded back to FP64).
void orcld_rk3(const f3d_params* P, int nsteps, double dt, double* U, double* Un, double* Q,
               const double* const m[9], const double* J) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using L = long double;
    std::vector<L> Ul(U, U + nc * 5), Unl(Un, Un + nc * 5), Ql(Q, Q + nc * 6), ml[9], Jl(J, J + nc);
    const L* mp[9];
    for (int a = 0; a < 9; a++) {
        ml[a].assign(m[a], m[a] + nc);
        mp[a] = ml[a].data();
    }
    Solver<L, L> s(*P, mp, Jl.data());
    for (int t = 0; t < nsteps; t++)
        s.rk3_step(L(dt), Ul.data(), Unl.data(), Ql.data());
    for (size_t i = 0; i < nc * 5; i++) {
        U[i] = (double)Ul[i];
        Un[i] = (double)Unl[i];
    }
    for (size_t i = 0; i < nc * 6; i++) Q[i] = (double)Ql[i];
}

void orc32_rhs(const f3d_params* P, const float* Q, const float* const m[9], const float* J, float* dUdt) {
    Solver<float, double> s(*P, m, J);
    s.rhs(Q, dUdt);
}
void orc32_rk3(const f3d_params* P, int nsteps, float dt, float* U, float* Un, float* Q, const float* const m[9],
               const float* J) {
    Solver<float, double> s(*P, m, J);
    for (int t = 0; t < nsteps; t++)
        s.rk3_step(dt, U, Un, Q);
}
void orc32_c2prim(const f3d_params* P, const float* U, float* Q) { c2prim<float>(*P, U, Q); }
void orc32_fill_ghosts(const f3d_params* P, float* Q, float* U) { fill_ghosts<float>(*P, Q, U); }
void orc32_prim2c(const f3d_params* P, const float* Q, float* U) { prim2c<float>(*P, Q, U); }

// ---- forward-mode derivative (dual numbers) -----------------------------------------
// JVP of the RHS as a function of the interior conserved state: U -> c2Prim -> ghost fill
// -> RHS. dU is the tangent of U (interior used); returns dUdt and its tangent.
void orc_rhs_jvp_u(const f3d_params* P, const double* U, const double* dU, const double* const m[9],
                   const double* J, double* dUdt, double* d_dUdt) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using D = Dual;
    std::vector<D> Ud(nc * 5), Qd(nc * 6, D(0.0)), Rd(nc * 5, D(0.0));
    for (size_t i = 0; i < nc * 5; i++) Ud[i] = D(U[i], dU[i]);
    std::vector<D> md[9], Jd(nc);
    const D* mp[9];
    for (int a = 0; a < 9; a++) {
        md[a].resize(nc);
        for (size_t i = 0; i < nc; i++) md[a][i] = D(m[a][i]);
        mp[a] = md[a].data();
    }
    for (size_t i = 0; i < nc; i++) Jd[i] = D(J[i]);
    c2prim<D>(*P, Ud.data(), Qd.data());
    fill_ghosts<D>(*P, Qd.data(), Ud.data());
    Solver<D, D> s(*P, mp, Jd.data());
    s.rhs(Qd.data(), Rd.data());
    for (size_t i = 0; i < nc * 5; i++) {
        dUdt[i] = Rd[i].v;
        d_dUdt[i] = Rd[i].d;
    }
}

// JVP of nsteps RK3 steps from the interior conserved state U0 (Q derived from U0 by
// c2Prim + ghost fill): returns U_final and its tangent.
void orc_rk3_jvp_u(const f3d_params* P, int nsteps, double dt, const double* U0, const double* dU0,
                   const double* const m[9], const double* J, double* U_out, double* dU_out) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using D = Dual;
    std::vector<D> Ud(nc * 5), Und(nc * 5, D(0.0)), Qd(nc * 6, D(0.0));
    for (size_t i = 0; i < nc * 5; i++) Ud[i] = D(U0[i], dU0[i]);
    std::vector<D> md[9], Jd(nc);
    const D* mp[9];
    for (int a = 0; a < 9; a++) {
        md[a].resize(nc);
        for (size_t i = 0; i < nc; i++) md[a][i] = D(m[a][i]);
        mp[a] = md[a].data();
    }
    for (size_t i = 0; i < nc; i++) Jd[i] = D(J[i]);
    c2prim<D>(*P, Ud.data(), Qd.data());
    fill_ghosts<D>(*P, Qd.data(), Ud.data());
    Solver<D, D> s(*P, mp, Jd.data());
    for (int t = 0; t < nsteps; t++)
        for (int st = 1; st <= 3; st++) s.rk3_stage(st, D(dt), Ud.data(), Und.data(), Qd.data());
    for (size_t i = 0; i < nc * 5; i++) {
        U_out[i] = Ud[i].v;
        dU_out[i] = Ud[i].d;
    }
}

// JVP of the RHS with respect to the metrics and J at a fixed ghost-filled Q (the metric
// tangents dm[9], dJ seed the dual numbers; |A| and A/|A| follow inside the solver).
void orc_rhs_jvp_m(const f3d_params* P, const double* Q, const double* const m[9], const double* const dm[9],
                   const double* J, const double* dJ, double* dUdt, double* d_dUdt) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using D = Dual;
    std::vector<D> Qd(nc * 6), Rd(nc * 5, D(0.0));
    for (size_t i = 0; i < nc * 6; i++) Qd[i] = D(Q[i]);
    std::vector<D> md[9], Jd(nc);
    const D* mp[9];
    for (int a = 0; a < 9; a++) {
        md[a].resize(nc);
        for (size_t i = 0; i < nc; i++) md[a][i] = D(m[a][i], dm[a][i]);
        mp[a] = md[a].data();
    }
    for (size_t i = 0; i < nc; i++) Jd[i] = D(J[i], dJ[i]);
    Solver<D, D> s(*P, mp, Jd.data());
    s.rhs(Qd.data(), Rd.data());
    for (size_t i = 0; i < nc * 5; i++) {
        dUdt[i] = Rd[i].v;
        d_dUdt[i] = Rd[i].d;
    }
}

// JVP of nsteps RK3 steps from a fixed U0 with respect to the metrics and J.
void orc_rk3_jvp_m(const f3d_params* P, int nsteps, double dt, const double* U0, const double* const m[9],
                   const double* const dm[9], const double* J, const double* dJ, double* U_out, double* dU_out) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using D = Dual;
    std::vector<D> Ud(nc * 5), Und(nc * 5, D(0.0)), Qd(nc * 6, D(0.0));
    for (size_t i = 0; i < nc * 5; i++) Ud[i] = D(U0[i]);
    std::vector<D> md[9], Jd(nc);
    const D* mp[9];
    for (int a = 0; a < 9; a++) {
        md[a].resize(nc);
        for (size_t i = 0; i < nc; i++) md[a][i] = D(m[a][i], dm[a][i]);
        mp[a] = md[a].data();
    }
    for (size_t i = 0; i < nc; i++) Jd[i] = D(J[i], dJ[i]);
    c2prim<D>(*P, Ud.data(), Qd.data());
    fill_ghosts<D>(*P, Qd.data(), Ud.data());
    Solver<D, D> s(*P, mp, Jd.data());
    for (int t = 0; t < nsteps; t++)
        for (int st = 1; st <= 3; st++) s.rk3_stage(st, D(dt), Ud.data(), Und.data(), Qd.data());
    for (size_t i = 0; i < nc * 5; i++) {
        U_out[i] = Ud[i].v;
        dU_out[i] = Ud[i].d;
    }
}

// ---- exact operation counts ------------------------------------------------------------
// Runs the RHS on counting scalars and returns the number of floating-point operations by
// class: out[0] add/sub, out[1] mul, out[2] div, out[3] sqrt, out[4] compare/abs/max.
// Fused multiply-add is not formed by the oracle, so a GPU FMA counts as one add + one mul.
void orc_rhs_opcount(const f3d_params* P, const double* Q, const double* const m[9], const double* J,
                     double* out) {
    Grid g(*P);
    const size_t nc = g.ncell();
    using C = Counted;
    std::vector<C> Qc(nc * 6), Rc(nc * 5, C(0.0));
    for (size_t i = 0; i < nc * 6; i++) Qc[i] = C(Q[i]);
    std::vector<C> mc[9], Jc(nc);
    const C* mp[9];
    for (int a = 0; a < 9; a++) {
        mc[a].resize(nc);
        for (size_t i = 0; i < nc; i++) mc[a][i] = C(m[a][i]);
        mp[a] = mc[a].data();
    }
    for (size_t i = 0; i < nc; i++) Jc[i] = C(J[i]);
    // metric norms are set-up work, not per-RHS work: build the solver before counting.
    // The counters are plain globals, so count on one thread.
    const int saved = omp_get_max_threads();
    omp_set_num_threads(1);
    Solver<C, C> s(*P, mp, Jc.data());
    opcount_reset();
    s.rhs(Qc.data(), Rc.data());
    opcount_read(out);
    omp_set_num_threads(saved);
}

}  // extern "C"
