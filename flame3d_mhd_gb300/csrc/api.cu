// api.cu — the extern "C" boundary of libflame3d_gpu.so (declared in include/flame3d_gpu.h).
//
// It replaces the @cuda launch sites of the reference's finite-difference path:
// flowAdvance (solver.jl:19-189), the RK3 stage loop (solver.jl:416-444), exchange_ghost
// (mpi.jl:2-103) and fillGhost (boundary.jl:151-156). Every entry point validates its
// arguments, launches asynchronously on the caller's stream and returns a status code.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <type_traits>

#include "f3d_kernels.cuh"

using namespace f3d;

namespace f3d {

// Branch every face takes when the thresholds leave no choice for a sensor value in
// [0, 3] (each directional term of schemes.jl:19-21 lies in [0,1] for positive p).
static int fixed_branch_of(const f3d_params& p) {
    const double top = 4.0;
    if (p.phi1 > top) return 0;
    if (p.phi1 <= 0.0 && p.phi2 > top) return 1;
    if (p.phi1 <= 0.0 && p.phi2 <= 0.0 && p.phi3 > top) return 2;
    if (p.phi1 <= 0.0 && p.phi2 <= 0.0 && p.phi3 <= 0.0) return 3;
    return -1;
}

int validate_params(const f3d_params& p, std::string& why) {
    if (p.ng != NG) { why = "ng must be 4"; return F3D_ERR_ARG; }
    if (p.nx < NG || p.ny < NG || p.nz < NG) { why = "each interior dimension must be >= 4"; return F3D_ERR_ARG; }
    if ((long long)p.nx > (1 << 20) || (long long)p.ny > 65535 - 8 || (long long)p.nz > 65535 - 8) {
        why = "grid too large for the launch shape"; return F3D_ERR_ARG;
    }
    const long long cells = (long long)(p.nx + 8) * (p.ny + 8) * (p.nz + 8);
    if (cells >= (1LL << 31)) { why = "grid too large (cell indices are 31-bit)"; return F3D_ERR_ARG; }
    if (!(p.gamma > 1.0) || !(p.rg > 0.0) || !(p.pr > 0.0) || !(p.c_s >= 0.0) || !(p.t_s >= 0.0)) {
        why = "gas constants out of range"; return F3D_ERR_ARG;
    }
    if (p.split_method < 0 || p.split_method > 3) { why = "unknown split_method"; return F3D_ERR_ARG; }
    if (p.character != 0 && p.character != 1) { why = "character must be 0 or 1"; return F3D_ERR_ARG; }
    if (p.viscous != 0 && p.viscous != 1) { why = "viscous must be 0 or 1"; return F3D_ERR_ARG; }
    if (p.precision < F3D_PREC_FP64 || p.precision > F3D_PREC_REF32) { why = "unknown precision"; return F3D_ERR_ARG; }
    if (p.precision == F3D_PREC_REF32 && (p.lts || p.filter)) {
        why = "the Float32 reference form has no local time stepping or filters";
        return F3D_ERR_UNSUPPORTED;
    }
    if (p.scheme < F3D_SCHEME_FDM || p.scheme > F3D_SCHEME_FVM_CONS) { why = "unknown scheme"; return F3D_ERR_ARG; }
    if (p.lts != 0 && p.lts != 1) { why = "lts must be 0 or 1"; return F3D_ERR_ARG; }
    if (p.adjoint_lean != 0 && p.adjoint_lean != 1) { why = "adjoint_lean must be 0 or 1"; return F3D_ERR_ARG; }
    if (p.lts && !(p.lts_cfl > 0.0)) { why = "lts_cfl must be > 0"; return F3D_ERR_ARG; }
    if (p.filter < F3D_FILTER_NONE || p.filter > F3D_FILTER_NONLINEAR) { why = "unknown filter"; return F3D_ERR_ARG; }
    if (p.filter && p.filter_interval < 1) { why = "filter_interval must be >= 1"; return F3D_ERR_ARG; }
    if (p.les < F3D_LES_NONE || p.les > F3D_LES_WALE) { why = "unknown les model"; return F3D_ERR_ARG; }
    if (p.scheme != F3D_SCHEME_FDM && p.precision != F3D_PREC_FP64) {
        why = "the finite-volume schemes are built for FP64";
        return F3D_ERR_UNSUPPORTED;
    }
    int iso_dirs = 0;
    for (int d = 0; d < 3; d++) {
        const f3d_bc &lo = p.bc[2 * d], &hi = p.bc[2 * d + 1];
        for (const f3d_bc* b : {&lo, &hi}) {
            if (b->kind == F3D_BC_INFLOW_PROFILE && p.precision == F3D_PREC_REF32) {
                why = "inflow-profile faces take FP64 profiles; the Float32 reference form has none";
                return F3D_ERR_UNSUPPORTED;
            }
            if (b->kind < 0 || b->kind > 5) { why = "unknown boundary kind"; return F3D_ERR_ARG; }
            if (b->kind == F3D_BC_DIRICHLET && !(b->rho > 0.0 && b->p > 0.0)) {
                why = "Dirichlet state needs rho > 0 and p > 0"; return F3D_ERR_ARG;
            }
            if (b->kind == F3D_BC_WALL_ISOTHERMAL && !(b->t_wall > 0.0)) {
                why = "isothermal wall needs t_wall > 0"; return F3D_ERR_ARG;
            }
        }
        if ((lo.kind == F3D_BC_PERIODIC) != (hi.kind == F3D_BC_PERIODIC)) {
            why = "periodic boundaries must be paired on both faces of a direction"; return F3D_ERR_ARG;
        }
        if (lo.kind == F3D_BC_WALL_ISOTHERMAL || hi.kind == F3D_BC_WALL_ISOTHERMAL) iso_dirs++;
    }
    if (iso_dirs > 1) { why = "isothermal walls on more than one direction are not supported"; return F3D_ERR_UNSUPPORTED; }
    return F3D_OK;
}

DevParams make_dev_params(const f3d_params& p) {
    DevParams d;
    std::memset(&d, 0, sizeof(d));
    d.nx = p.nx; d.ny = p.ny; d.nz = p.nz;
    d.nxt = p.nx + 2 * NG; d.nyt = p.ny + 2 * NG; d.nzt = p.nz + 2 * NG;
    d.plane = (long long)d.nxt * d.nyt * d.nzt;
    d.dnxt = make_fastdiv((unsigned)d.nxt); d.dnyt = make_fastdiv((unsigned)d.nyt);
    d.dnx = make_fastdiv((unsigned)p.nx); d.dny = make_fastdiv((unsigned)p.ny);
    d.dvxt = make_fastdiv((unsigned)(d.nxt - 4)); d.dvyt = make_fastdiv((unsigned)(d.nyt - 4));
    d.gamma = p.gamma; d.rg = p.rg;
    d.cp = p.cp != 0.0 ? p.cp : p.rg * p.gamma / (p.gamma - 1.0);
    d.c_s = p.c_s; d.t_s = p.t_s; d.pr = p.pr;
    d.gm1 = p.gamma - 1.0;
    d.inv_rg = 1.0 / p.rg;
    d.grg = p.gamma * p.rg;
    d.eps_clamp = p.clamp_eps != 0.0 ? p.clamp_eps : 1.1920928955078125e-07;
    d.phi1 = p.phi1; d.phi2 = p.phi2; d.phi3 = p.phi3;
    const double up7[7] = {-3.0 / 420, 25.0 / 420, -101.0 / 420, 319.0 / 420, 214.0 / 420, -38.0 / 420, 4.0 / 420};
    const double cd6[7] = {0.0, 1.0 / 60, -2.0 / 15, 37.0 / 60, 37.0 / 60, -2.0 / 15, 1.0 / 60};
    for (int m = 0; m < 7; m++) d.lin[m] = up7[m] * p.linear_phi + cd6[m] * (1.0 - p.linear_phi);
    d.split = p.split_method; d.character = p.character; d.viscous = p.viscous;
    d.precision = p.precision;
    d.lts = p.lts;
    d.les = p.les;
    d.fixed_branch = fixed_branch_of(p);
    const double th[3] = {p.phi1, p.phi2, p.phi3};
    for (int k = 0; k < 3; k++) {
        unsigned long long b = 0;
        if (th[k] > 0.0) std::memcpy(&b, &th[k], 8);
        d.phib[k] = b;
    }
    auto fill = [&](auto& c) {
        using R = std::remove_reference_t<decltype(c.gamma)>;
        c.gamma = (R)p.gamma; c.rg = (R)p.rg; c.grg = (R)d.grg; c.gm1 = (R)d.gm1;
        c.inv_gm1 = (R)(1.0 / d.gm1); c.inv_2g = (R)(1.0 / (2.0 * p.gamma)); c.two_gm1 = (R)(2.0 * d.gm1);
        c.w2c = (R)((3.0 - p.gamma) / (2.0 * d.gm1));
        c.c_s = (R)d.c_s; c.t_s = (R)d.t_s; c.cp = (R)d.cp; c.pr = (R)d.pr;
        c.cp_pr = (R)(d.cp / d.pr);
        c.phi1 = (R)p.phi1; c.phi2 = (R)p.phi2; c.phi3 = (R)p.phi3;
        for (int m = 0; m < 7; m++) c.lin[m] = (R)d.lin[m];
    };
    fill(d.cd);
    fill(d.cf);
    d.ref32 = p.precision == F3D_PREC_REF32;
    d.g32 = (float)p.gamma;
    d.rg32 = (float)p.rg;
    d.gm1_32 = d.g32 - 1.0f;
    d.eps32 = (float)d.eps_clamp;
    if (d.ref32) {  // the reference's Float32 constants, derived in Float32 as its code does
        Cst<float>& c = d.cf;
        const float g = d.g32, rg = d.rg32, gm1 = d.gm1_32;
        c.gamma = g; c.rg = rg; c.gm1 = gm1; c.grg = g * rg;
        c.inv_gm1 = 1.0f / gm1; c.inv_2g = 1.0f / (2.0f * g); c.two_gm1 = 2.0f * gm1;
        c.w2c = (3.0f - g) / (2.0f * gm1);
        c.cp = p.cp != 0.0 ? (float)p.cp : rg * g / gm1;
        c.cp_pr = c.cp / c.pr;
        const float lp = (float)p.linear_phi;
        for (int m = 0; m < 7; m++) c.lin[m] = (float)up7[m] * lp + (float)cd6[m] * (1.0f - lp);
    }
    for (int f = 0; f < 6; f++) {
        const f3d_bc& b = p.bc[f];
        d.bc[f].kind = b.kind;
        d.bc[f].rho = b.rho; d.bc[f].u = b.u; d.bc[f].v = b.v; d.bc[f].w = b.w; d.bc[f].p = b.p;
        d.bc[f].T = b.kind == F3D_BC_DIRICHLET ? b.p / (b.rho * p.rg) : 0.0;
        d.bc[f].t_wall = b.t_wall;
    }
    return d;
}

}  // namespace f3d

// Per-launch event recording for f3d_profile_step.
struct Prof {
    static constexpr int kMax = 64;
    cudaEvent_t ev[kMax];
    int kind[kMax];
    int nl[kMax];  // kernels launched since the previous mark
    int n = 0;
};

struct f3d_ctx {
    f3d_params params;
    DevParams dp;
    int device = 0;
    std::string err;
    const double* m[9] = {};
    const double* J = nullptr;
    bool metrics_set = false;
    // scratch (one allocation)
    void* slab = nullptr;
    size_t slab_bytes = 0;
    double* S[3] = {};
    double* Ah[9] = {};
    double* csnd = nullptr;
    double* phi = nullptr;
    double* acc = nullptr;
    double* Fv[3] = {};
    // finite-volume schemes: face normals and areas (nx, ny, nz, area per direction) and
    // the conserved state f3d_rhs reconstructs from (prim2c of its Q)
    double* geo[12] = {};
    double* Ufv = nullptr;
    bool coords_set = false;
    // local time step (lts) and the shock-capturing filter's sensor; steps done by
    // f3d_rk3_steps (the filter runs after every filter_interval-th)
    double* dtl = nullptr;
    double* sc = nullptr;
    long long tt = 0;
    void* extra = nullptr;
    // mixed precision: FP32 copies and FP32 intermediates
    float* Q32 = nullptr;
    MetricPtrs32 m32 = {};
    float* phi32 = nullptr;
    float* acc32 = nullptr;
    float* acc32b = nullptr;  // mixed form: the eta sweep's differences (summed in FP64 by the last)
    float* Fv32[3] = {};
    double* dscalar = nullptr;  // 8 bytes for reductions
    unsigned* kstat = nullptr;  // kernel status word (bit 0: a TMA tile wait gave up)
    unsigned* tile_ctr = nullptr;  // next-tile counters of the TMA sweeps
    // mixed form: the TMA-staged sweeps and their tensor maps (three directions)
    bool use_tma = false;
    void* tma_maps = nullptr;
    // the last sweep's staged Phase C maps, encoded for the arrays of epi_key (U, Un, J)
    void* epi_maps = nullptr;
    const void* epi_key[3] = {};
    Prof* prof = nullptr;
    // adjoint scratch, allocated by the first VJP call
    void* adj_slab = nullptr;
    double *Qb = nullptr, *Lt = nullptr, *U1 = nullptr, *U2 = nullptr, *Xb = nullptr, *Yb = nullptr;
    double *Qst[3] = {}, *cst_[3] = {}, *phst[3] = {};  // Q, sound speed and sensor of the stage states
    double *Fvb[3] = {}, *gb = nullptr;
    // metric and Jacobian cotangents (borrowed; f3d_set_metrics_cotangent) and the forward
    // RHS of the first two stage states kept for the Jacobian's term (10 arrays, owned)
    double* mbar[9] = {};
    double* Jbar = nullptr;
    double* lsave = nullptr;
    // CUDA graph of one RK3 step, keyed by its arguments
    cudaGraphExec_t step_graph = nullptr;
    const void* g_key[4] = {};
    double g_dt = 0.0;
};

namespace {

enum KernelKind { K_SOUND = 0, K_SENSOR, K_VISCOUS, K_SWEEP_X, K_SWEEP_Y, K_SWEEP_Z, K_PRIM_FILL, K_STAGE_UPDATE,
                  K_NKIND };
const char* kKernelNames[K_NKIND] = {"sound_speed", "shock_sensor", "viscous_flux", "sweep_xi",
                                     "sweep_eta", "sweep_zeta", "prim_ghost_fill", "stage_update"};

void mark(f3d_ctx* ctx, int kind, cudaStream_t st, int launches = 1) {
    Prof* p = ctx->prof;
    if (p && p->n < Prof::kMax) {
        cudaEventRecord(p->ev[p->n], st);
        p->nl[p->n] = launches;
        p->kind[p->n++] = kind;
    }
}

int fail(f3d_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->err = msg;
    return code;
}

int cuda_fail(f3d_ctx* ctx, cudaError_t e, const char* where) {
    return fail(ctx, F3D_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define F3D_CUDA(ctx, call)                                              \
    do {                                                                 \
        cudaError_t e_ = (call);                                         \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);      \
    } while (0)

bool aligned(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int check_ptrs(f3d_ctx* ctx, std::initializer_list<const void*> ps) {
    for (const void* p : ps) {
        if (!p) return fail(ctx, F3D_ERR_ARG, "null array pointer");
        if (!aligned(p)) return fail(ctx, F3D_ERR_ALIGN, "array pointer not 16-byte aligned");
    }
    return F3D_OK;
}

// need_state: a compute call (metrics set, and every inflow-profile face has its profile).
// The FP64-array entries refuse an F3D_PREC_REF32 context (its arrays are Float32: the
// *_f32 entries), and those refuse the other contexts (check_ctx32).
int check_ctx(f3d_ctx* ctx, bool need_state, bool f32_entry = false) {
    if (!ctx) return F3D_ERR_ARG;
    if (ctx->dp.ref32 && !f32_entry)
        return fail(ctx, F3D_ERR_ARG, "an F3D_PREC_REF32 context takes Float32 arrays: use the _f32 entries");
    if (!ctx->dp.ref32 && f32_entry)
        return fail(ctx, F3D_ERR_ARG, "the _f32 entries need an F3D_PREC_REF32 context");
    if (need_state && !ctx->metrics_set) return fail(ctx, F3D_ERR_STATE, "metrics not set (call f3d_set_metrics)");
    if (need_state && ctx->params.scheme != F3D_SCHEME_FDM && !ctx->coords_set)
        return fail(ctx, F3D_ERR_STATE, "coordinates not set (call f3d_set_coordinates)");
    for (int f = 0; f < 6 && need_state; f++)
        if (ctx->params.bc[f].kind == F3D_BC_INFLOW_PROFILE && !ctx->dp.prof[f])
            return fail(ctx, F3D_ERR_STATE, "inflow profile not set (call f3d_set_inflow_profile)");
    if (cudaSetDevice(ctx->device) != cudaSuccess) return fail(ctx, F3D_ERR_CUDA, "cudaSetDevice failed");
    return F3D_OK;
}

bool mixed(const f3d_ctx* ctx) { return ctx->dp.precision == F3D_PREC_MIXED; }
int check_ctx32(f3d_ctx* ctx, bool need_state) { return check_ctx(ctx, need_state, true); }

// Forget the captured RK3 step: its kernels hold pointers and parameters by value.
void drop_step_graph(f3d_ctx* ctx) {
    if (ctx->step_graph) cudaGraphExecDestroy(ctx->step_graph);
    ctx->step_graph = nullptr;
}

SweepArgs sweep_args(f3d_ctx* ctx, int dir, const double* Q, bool hybrid, const double* phi_override = nullptr,
                     const float* Q32 = nullptr) {
    SweepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.P = ctx->dp;
    a.J = ctx->J;
    a.kstat = ctx->kstat;
    a.tile_ctr = ctx->tile_ctr;
    if (mixed(ctx) || ctx->dp.ref32) {
        a.fp32 = 1;
        a.Q = ctx->dp.ref32 ? Q32 : ctx->Q32;
        for (int n = 0; n < 3; n++) {
            a.A[n] = ctx->m32.A[3 * dir + n];
            a.Ah[n] = ctx->m32.H[3 * dir + n];
        }
        a.S = ctx->m32.S[dir];
        a.phi = hybrid ? ctx->phi32 : nullptr;
        a.Fv = ctx->params.viscous ? ctx->Fv32[dir] : nullptr;
        return a;
    }
    a.Q = Q;
    a.csnd = ctx->csnd;
    for (int n = 0; n < 3; n++) {
        a.A[n] = ctx->m[3 * dir + n];
        a.Ah[n] = ctx->Ah[3 * dir + n];
    }
    a.S = ctx->S[dir];
    a.phi = hybrid ? (phi_override ? phi_override : ctx->phi) : nullptr;
    a.Fv = ctx->params.viscous ? ctx->Fv[dir] : nullptr;
    return a;
}

// Sensor, viscous fluxes and the three sweeps. last.out_mode is OUT_RHS or OUT_STAGE.
// fill_current: the previous stage's primitive fill already wrote what the sweeps read besides
// Q (mixed precision: the FP32 copy of Q; FP64: the sound speed), so it is not made again.
// Finite-volume RHS (FVM.jl): sensor, viscous fluxes, three face sweeps reconstructing the
// conserved state (the stage's U, or prim2c(Q) for f3d_rhs) and, for a stage, the RK update
// after the last sweep (the sweeps read U, so it cannot be updated inside them).
int run_rhs_fvm(f3d_ctx* ctx, const double* Q, double* acc, const SweepArgs& last, cudaStream_t st) {
    const DevParams& P = ctx->dp;
    const bool hybrid = P.fixed_branch < 0;
    const bool stage = last.out_mode == OUT_STAGE;
    const double* U = stage ? last.U : ctx->Ufv;
    if (!stage) F3D_CUDA(ctx, launch_prim2c(P, Q, ctx->Ufv, st));
    if (hybrid) {
        F3D_CUDA(ctx, launch_sensor(P, Q, ctx->phi, st));
        mark(ctx, K_SENSOR, st);
    }
    if (ctx->params.viscous) {
        F3D_CUDA(ctx, launch_viscous(P, Q, ctx->m, ctx->J, ctx->Fv[0], ctx->Fv[1], ctx->Fv[2], st));
        mark(ctx, K_VISCOUS, st);
    }
    const bool eigen = ctx->params.scheme == F3D_SCHEME_FVM_EIGEN;
    for (int d = 0; d < 3; d++) {
        SweepArgs a = sweep_args(ctx, d, Q, hybrid);
        a.acc = acc;
        a.out = acc;
        a.out_mode = d == 0 ? OUT_SET : OUT_ADD;
        if (d == 2 && !stage) {
            a.out_mode = last.out_mode;
            a.out = last.out;
        }
        F3D_CUDA(ctx, launch_fvm_sweep(d, eigen, a, U, ctx->geo, st));
        mark(ctx, K_SWEEP_X + d, st);
    }
    if (stage) {
        F3D_CUDA(ctx, launch_stage_update(P, acc, ctx->J, last.dt, last.U, last.Un, last.stage1_copy, last.combine,
                                          last.ca, last.cb, st, last.dtl));
        mark(ctx, K_STAGE_UPDATE, st);
    }
    return F3D_OK;
}

int run_rhs(f3d_ctx* ctx, const double* Q, double* acc, SweepArgs last, cudaStream_t st, bool fill_current = false) {
    if (ctx->params.scheme != F3D_SCHEME_FDM) return run_rhs_fvm(ctx, Q, acc, last, st);
    const DevParams& P = ctx->dp;
    const bool hybrid = P.fixed_branch < 0;
    const bool mx = mixed(ctx);
    if (mx) {
        if (!fill_current) {
            F3D_CUDA(ctx, launch_to_f32(Q, ctx->Q32, 6 * P.plane, st));
            mark(ctx, K_SOUND, st);
        }
        if (hybrid) {
            F3D_CUDA(ctx, launch_sensor32(P, ctx->Q32, ctx->phi32, st));
            mark(ctx, K_SENSOR, st);
        }
        if (ctx->params.viscous) {
            const float* m32[9];
            for (int n = 0; n < 9; n++) m32[n] = ctx->m32.A[n];
            F3D_CUDA(ctx, launch_viscous32(P, ctx->Q32, m32, ctx->m32.J, ctx->Fv32[0], ctx->Fv32[1], ctx->Fv32[2], st));
            mark(ctx, K_VISCOUS, st);
        }
    } else {
        if (!fill_current) {
            F3D_CUDA(ctx, launch_sound(P, Q, ctx->csnd, st));
            mark(ctx, K_SOUND, st);
        }
        if (hybrid) {
            F3D_CUDA(ctx, launch_sensor(P, Q, ctx->phi, st));
            mark(ctx, K_SENSOR, st);
        }
        if (ctx->params.viscous) {
            F3D_CUDA(ctx, launch_viscous(P, Q, ctx->m, ctx->J, ctx->Fv[0], ctx->Fv[1], ctx->Fv[2], st));
            mark(ctx, K_VISCOUS, st);
        }
    }
    if (ctx->use_tma) F3D_CUDA(ctx, cudaMemsetAsync(ctx->tile_ctr, 0, 3 * sizeof(unsigned), st));
    for (int d = 0; d < 3; d++) {
        SweepArgs a = sweep_args(ctx, d, Q, hybrid);
        a.acc = mx ? (void*)ctx->acc32 : (void*)acc;
        if (d == 0) a.out_mode = OUT_SET;
        else if (d == 1) {
            // mixed: the eta differences go to their own array; the last sweep sums in FP64
            a.out_mode = mx ? OUT_SET : OUT_ADD;
            if (mx) a.acc = ctx->acc32b;
        } else {
            if (mx) a.acc2 = ctx->acc32b;
            a.out_mode = last.out_mode;
            a.out = last.out;
            a.U = last.U;
            a.Un = last.Un;
            a.dt = last.dt;
            a.ca = last.ca;
            a.cb = last.cb;
            a.combine = last.combine;
            a.stage1_copy = last.stage1_copy;
            a.dtl = last.dtl;
        }
        if (ctx->use_tma) {
            // the last sweep stages its Phase C inputs too (not with a per-cell time step)
            const void* epi = nullptr;
            if (d == 2 && !a.dtl && (a.out_mode == OUT_RHS || a.out_mode == OUT_STAGE)) {
                const double* Ue = a.out_mode == OUT_STAGE ? a.U : nullptr;
                const double* Une = a.out_mode == OUT_STAGE ? a.Un : nullptr;
                const void* key[3] = {Ue, Une, ctx->J};
                if (std::memcmp(key, ctx->epi_key, sizeof(key)) != 0) {
                    ctx->epi_key[0] = nullptr;  // invalid until encoded
                    F3D_CUDA(ctx, make_epi_maps(ctx->dp, ctx->acc32, ctx->acc32b, ctx->J, Ue, Une, ctx->epi_maps));
                    std::memcpy(ctx->epi_key, key, sizeof(key));
                }
                epi = ctx->epi_maps;
            }
            F3D_CUDA(ctx, launch_sweep_tma(d, a, ctx->tma_maps, epi, st));
        } else {
            F3D_CUDA(ctx, launch_sweep(d, a, st));
        }
        mark(ctx, K_SWEEP_X + d, st);
    }
    return F3D_OK;
}

// The stage's primitive fill also writes the FP32 copy of Q (mixed precision) or the sound
// speed (FP64 finite differences) that the next stage's sweeps read.
int run_stage(f3d_ctx* ctx, int stage, double dt, double* U, double* Un, double* Q, cudaStream_t st,
              bool fill_current = false) {
    SweepArgs last;
    std::memset(&last, 0, sizeof(last));
    last.out_mode = OUT_STAGE;
    last.U = U;
    last.Un = Un;
    last.dt = dt;
    last.stage1_copy = stage == 1;
    last.combine = stage != 1;
    last.ca = stage == 2 ? 0.25 : 2.0 / 3.0;  // utils.jl:57-70 via solver.jl:433-435
    last.cb = stage == 2 ? 0.75 : 1.0 / 3.0;
    if (ctx->params.lts) {  // compute_dt at the first stage only (solver.jl:418-421), div_LTS in all
        if (stage == 1)
            F3D_CUDA(ctx, launch_local_dt(ctx->dp, Q, ctx->m, ctx->J, ctx->params.lts_cfl, ctx->dtl, st));
        last.dtl = ctx->dtl;
    }
    int rc = run_rhs(ctx, Q, ctx->acc, last, st, fill_current);
    if (rc) return rc;
    const bool mx = mixed(ctx), fdm64 = !mx && ctx->params.scheme == F3D_SCHEME_FDM;
    F3D_CUDA(ctx, launch_prim_fill(ctx->dp, U, Q, U, fdm64 ? ctx->csnd : nullptr, 0, st, mx ? ctx->Q32 : nullptr));
    mark(ctx, K_PRIM_FILL, st, 2);  // interior and ghost passes
    return F3D_OK;
}

// ---- discrete adjoint ------------------------------------------------------------------
// The explicit filters after every filter_interval-th step (solver.jl:446-470): per
// direction Un = U, then U = filter(Un) at interior cells. Q is left as it is, as the
// reference leaves it until the next stage recomputes it.
int apply_filter(f3d_ctx* ctx, double* U, double* Un, const double* Q, cudaStream_t st) {
    const f3d_params& p = ctx->params;
    for (int d = 0; d < 3; d++) {
        F3D_CUDA(ctx, cudaMemcpyAsync(Un, U, (size_t)ctx->dp.plane * 5 * sizeof(double), cudaMemcpyDeviceToDevice, st));
        F3D_CUDA(ctx, launch_filter_dir(ctx->dp, d, p.filter, p.filter_s0, p.filter_rth, Q, U, Un, ctx->sc, st));
    }
    return F3D_OK;
}

int adjoint_supported(f3d_ctx* ctx) {
    if (mixed(ctx)) return fail(ctx, F3D_ERR_UNSUPPORTED, "the adjoint is built for the FP64 form");
    if (ctx->params.lts || ctx->params.filter || ctx->params.les)
        return fail(ctx, F3D_ERR_UNSUPPORTED, "the adjoint has no local time stepping, filters or LES");
    if (ctx->params.scheme != F3D_SCHEME_FDM)
        return fail(ctx, F3D_ERR_UNSUPPORTED, "the adjoint is built for the finite-difference scheme");
    return F3D_OK;
}

int adjoint_alloc(f3d_ctx* ctx) {
    if (ctx->adj_slab) return F3D_OK;
    const size_t nc = (size_t)ctx->dp.plane;
    const size_t nv = (size_t)(ctx->params.nx + 4) * (ctx->params.ny + 4) * (ctx->params.nz + 4);
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b1 = up(nc * 8);
    const size_t bv = up(nv * 8);
    const int ncache = ctx->params.adjoint_lean ? 1 : 3;
    size_t total = b1 * (6 + 5 * 5 + 8 * ncache) + (ctx->params.viscous ? bv * (12 + 12) : 0);
    cudaError_t e = cudaMalloc(&ctx->adj_slab, total);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc (adjoint scratch)");
    char* q = (char*)ctx->adj_slab;
    ctx->Qb = (double*)q; q += 6 * b1;
    ctx->Lt = (double*)q; q += 5 * b1;
    ctx->U1 = (double*)q; q += 5 * b1;
    ctx->U2 = (double*)q; q += 5 * b1;
    ctx->Xb = (double*)q; q += 5 * b1;
    ctx->Yb = (double*)q; q += 5 * b1;
    for (int k = 0; k < 3; k++) {  // lean: the three stages share one cache
        if (k < ncache) {
            ctx->Qst[k] = (double*)q; q += 6 * b1;
            ctx->cst_[k] = (double*)q; q += b1;
            ctx->phst[k] = (double*)q; q += b1;
        } else {
            ctx->Qst[k] = ctx->Qst[0]; ctx->cst_[k] = ctx->cst_[0]; ctx->phst[k] = ctx->phst[0];
        }
    }
    if (ctx->params.viscous) {
        for (int d = 0; d < 3; d++) { ctx->Fvb[d] = (double*)q; q += 4 * bv; }
        ctx->gb = (double*)q;
    }
    e = cudaMemset(ctx->adj_slab, 0, total);
    if (e == cudaSuccess) e = adjoint_configure();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "adjoint set-up");
    return F3D_OK;
}

// Q (ghost-filled c2Prim(U)), split sound speed and sensor of a state U, into the given
// buffers: everything the RHS and its VJP need from the forward state.
int prep_state(f3d_ctx* ctx, const double* U, double* Q, double* csnd, double* phi, cudaStream_t st) {
    F3D_CUDA(ctx, launch_prim_fill(ctx->dp, U, Q, nullptr, csnd, 0, st));
    if (ctx->dp.fixed_branch < 0) F3D_CUDA(ctx, launch_sensor(ctx->dp, Q, phi, st));
    return F3D_OK;
}

// L at interior cells into out, from a prepared state (the sweeps only)
int rhs_prepared(f3d_ctx* ctx, const double* Q, const double* csnd, const double* phi, double* out, cudaStream_t st) {
    const DevParams& P = ctx->dp;
    const bool hybrid = P.fixed_branch < 0;
    if (ctx->params.viscous) F3D_CUDA(ctx, launch_viscous(P, Q, ctx->m, ctx->J, ctx->Fv[0], ctx->Fv[1], ctx->Fv[2], st));
    for (int d = 0; d < 3; d++) {
        SweepArgs a = sweep_args(ctx, d, Q, hybrid, phi);
        a.csnd = csnd;
        a.acc = out;
        a.out = out;
        a.out_mode = d == 0 ? OUT_SET : (d == 1 ? OUT_ADD : OUT_RHS);
        F3D_CUDA(ctx, launch_sweep(d, a, st));
    }
    return F3D_OK;
}

// out = beta out + alpha (dL/dU)^T Lb at interior cells, for the state U prepared in Q/csnd/phi
// With metric cotangents set (ctx->mbar) the metric and Jacobian cotangents are accumulated
// too, scaled by alpha; Lfwd is the forward RHS of the state (for the Jacobian's L = J D).
int rhs_vjp_prepared(f3d_ctx* ctx, const double* U, const double* Q, const double* csnd, const double* phi,
                     const double* Lb, double* out, double alpha, double beta, cudaStream_t st,
                     const double* Lfwd = nullptr) {
    const bool mbar = ctx->mbar[0] != nullptr;
    const DevParams& P = ctx->dp;
    const bool hybrid = P.fixed_branch < 0;
    F3D_CUDA(ctx, cudaMemsetAsync(ctx->Qb, 0, (size_t)P.plane * 6 * sizeof(double), st));
    for (int d = 0; d < 3; d++) {
        AdjArgs a;
        std::memset(&a, 0, sizeof(a));
        a.P = P;
        a.Q = Q;
        a.csnd = csnd;
        for (int n = 0; n < 3; n++) {
            a.A[n] = ctx->m[3 * d + n];
            a.Ah[n] = ctx->Ah[3 * d + n];
        }
        a.S = ctx->S[d];
        a.phi = hybrid ? phi : nullptr;
        a.J = ctx->J;
        a.Lb = Lb;
        a.Qb = ctx->Qb;
        if (mbar) {
            for (int n = 0; n < 3; n++) a.mb[n] = ctx->mbar[3 * d + n];
            a.mscale = alpha;
        }
        F3D_CUDA(ctx, launch_sweep_vjp(d, a, st));
    }
    if (ctx->params.viscous)
        F3D_CUDA(ctx, launch_viscous_vjp(P, Q, ctx->m, ctx->J, Lb, ctx->Fvb, ctx->gb, ctx->Qb, st,
                                         mbar ? ctx->mbar : nullptr, ctx->Jbar, alpha));
    if (mbar) {
        if (!Lfwd) return fail(ctx, F3D_ERR_STATE, "metric cotangents need the forward RHS of the state");
        F3D_CUDA(ctx, launch_jbar(P, Lb, Lfwd, ctx->J, ctx->Jbar, alpha, st));
    }
    F3D_CUDA(ctx, launch_fill_vjp(P, Q, ctx->Qb, alpha, st));
    F3D_CUDA(ctx, launch_c2prim_vjp(P, U, ctx->Qb, out, alpha, beta, st));
    return F3D_OK;
}

// ---- F3D_PREC_REF32: the reference's Float32 form on the caller's Float32 arrays ----------
// Sensor, viscous fluxes and the three FP32 sweeps from the Float32 Q; the last sweep
// writes the Float32 RHS (OUT_RHS) or applies the Float32 RK update (OUT_STAGE).
int run_rhs32(f3d_ctx* ctx, const float* Q, const SweepArgs& last, cudaStream_t st) {
    const DevParams& P = ctx->dp;
    const bool hybrid = P.fixed_branch < 0;
    if (hybrid) {
        F3D_CUDA(ctx, launch_sensor32(P, Q, ctx->phi32, st));
        mark(ctx, K_SENSOR, st);
    }
    if (ctx->params.viscous) {
        const float* m32[9];
        for (int n = 0; n < 9; n++) m32[n] = ctx->m32.A[n];
        F3D_CUDA(ctx, launch_viscous32(P, Q, m32, ctx->m32.J, ctx->Fv32[0], ctx->Fv32[1], ctx->Fv32[2], st));
        mark(ctx, K_VISCOUS, st);
    }
    for (int d = 0; d < 3; d++) {
        SweepArgs a = sweep_args(ctx, d, nullptr, hybrid, nullptr, Q);
        a.acc = ctx->acc32;
        a.out_mode = d == 0 ? OUT_SET : (d == 1 ? OUT_ADD : last.out_mode);
        if (d == 2) {
            a.J32 = ctx->m32.J;
            a.out32 = last.out32;
            a.U32 = last.U32;
            a.Un32 = last.Un32;
            a.dt32 = last.dt32;
            a.ca32 = last.ca32;
            a.cb32 = last.cb32;
            a.combine = last.combine;
            a.stage1_copy = last.stage1_copy;
        }
        F3D_CUDA(ctx, launch_sweep(d, a, st));
        mark(ctx, K_SWEEP_X + d, st);
    }
    return F3D_OK;
}

// solver.jl:416-444 in Float32: U += dt J L, linComb, c2Prim, ghost fill
int run_stage32(f3d_ctx* ctx, int stage, float dt, float* U, float* Un, float* Q, cudaStream_t st) {
    SweepArgs last;
    std::memset(&last, 0, sizeof(last));
    last.out_mode = OUT_STAGE;
    last.U32 = U;
    last.Un32 = Un;
    last.dt32 = dt;
    last.stage1_copy = stage == 1;
    last.combine = stage != 1;
    last.ca32 = stage == 2 ? 0.25f : 2.0f / 3.0f;  // the Float32 weights of utils.jl:57-70
    last.cb32 = stage == 2 ? 0.75f : 1.0f / 3.0f;
    int rc = run_rhs32(ctx, Q, last, st);
    if (rc) return rc;
    F3D_CUDA(ctx, launch_prim_fill32(ctx->dp, U, Q, U, 0, st));
    mark(ctx, K_PRIM_FILL, st, 2);
    return F3D_OK;
}

}  // namespace

extern "C" {

int f3d_version(void) { return F3D_VERSION; }

int f3d_default_params(int nx, int ny, int nz, f3d_params* p) {
    if (!p) return F3D_ERR_ARG;
    std::memset(p, 0, sizeof(*p));
    p->nx = nx; p->ny = ny; p->nz = nz; p->ng = NG;
    p->gamma = 1.4; p->rg = 287.0; p->cp = 0.0; p->c_s = 1.458e-6; p->t_s = 110.4; p->pr = 0.72;  // run.jl:8-13
    p->phi1 = 0.05; p->phi2 = 1.0; p->phi3 = 10.0; p->linear_phi = 1.0;                          // run.jl:70-73
    p->clamp_eps = 0.0;
    p->split_method = F3D_SPLIT_SW; p->character = 1; p->viscous = 1;                            // run.jl:61,68,69
    p->precision = F3D_PREC_FP64;
    p->lts_cfl = 0.5;                                                                           // run.jl:22
    p->filter_interval = 100; p->filter_rth = 1e-5; p->filter_s0 = 1.0;                          // run.jl:52-54
    // boundary.jl: Dirichlet free stream inlet, zero-gradient outlet, adiabatic no-slip wall,
    // Dirichlet far field, periodic span.
    f3d_bc fs;
    std::memset(&fs, 0, sizeof(fs));
    fs.kind = F3D_BC_DIRICHLET; fs.rho = 1.0; fs.u = 0.5; fs.v = 0.0; fs.w = 0.0; fs.p = 1.0 / 1.4;
    p->bc[0] = fs;
    p->bc[1].kind = F3D_BC_ZERO_GRADIENT;
    p->bc[2].kind = F3D_BC_WALL_ADIABATIC;
    p->bc[3] = fs;
    p->bc[4].kind = F3D_BC_PERIODIC;
    p->bc[5].kind = F3D_BC_PERIODIC;
    return F3D_OK;
}

int f3d_create(const f3d_params* p, f3d_ctx** out) {
    if (!p || !out) return F3D_ERR_ARG;
    *out = nullptr;
    std::string why;
    int rc = validate_params(*p, why);
    if (rc) {
        std::fprintf(stderr, "f3d_create: %s\n", why.c_str());
        return rc;
    }
    f3d_ctx* ctx = new (std::nothrow) f3d_ctx();  // no exception crosses the C ABI
    if (!ctx) return F3D_ERR_CUDA;
    ctx->params = *p;
    ctx->dp = make_dev_params(*p);
    if (cudaGetDevice(&ctx->device) != cudaSuccess) { delete ctx; return F3D_ERR_CUDA; }
    const size_t nplane = (size_t)ctx->dp.plane;
    if (p->lts || p->filter == F3D_FILTER_NONLINEAR) {  // local dt, filter sensor (zero outside the interior)
        const size_t eb = nplane * sizeof(double) * 2;
        if (cudaMalloc(&ctx->extra, eb) != cudaSuccess || cudaMemset(ctx->extra, 0, eb) != cudaSuccess) {
            if (ctx->extra) cudaFree(ctx->extra);
            delete ctx;
            std::fprintf(stderr, "f3d_create: cudaMalloc of the step-component scratch failed\n");
            return F3D_ERR_CUDA;
        }
        ctx->dtl = (double*)ctx->extra;
        ctx->sc = ctx->dtl + nplane;
    }
    const size_t nc = (size_t)ctx->dp.plane;
    const size_t nv = (size_t)(p->nx + 4) * (p->ny + 4) * (p->nz + 4);
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const bool mx = p->precision != F3D_PREC_FP64;  // FP32 sweeps: the mixed and reference forms
    const bool r32 = p->precision == F3D_PREC_REF32;
    size_t total = 256;
    const bool fvm = p->scheme != F3D_SCHEME_FDM;
    if (!mx) {  // S(3) + A/|A|(9) + sound speed + phi + acc(5) [+ viscous 12] [+ FVM 12 + 5]
        total += up(nc * 8) * (3 + 9 + 1 + 1 + 5 + (fvm ? 17 : 0)) + (p->viscous ? 3 * up(nv * 4 * 8) : 0);
    } else {    // [Q32(6) + A32(9) + J32 + acc32b(5), mixed only] + H32(9) + S32(3) + phi32 + acc32(5) [+ viscous 12]
        total += up(nc * 4) * ((r32 ? 0 : 21) + 9 + 3 + 1 + 5) + (p->viscous ? 3 * up(nv * 4 * 4) : 0);
    }
    cudaError_t e = cudaMalloc(&ctx->slab, total);
    if (e != cudaSuccess) {
        if (ctx->extra) cudaFree(ctx->extra);
        delete ctx;
        std::fprintf(stderr, "f3d_create: cudaMalloc(%zu) failed: %s\n", total, cudaGetErrorString(e));
        return F3D_ERR_CUDA;
    }
    ctx->slab_bytes = total;
    char* q = (char*)ctx->slab;
    size_t phi_bytes;
    if (!mx) {
        const size_t b1 = up(nc * 8);
        for (int d = 0; d < 3; d++) { ctx->S[d] = (double*)q; q += b1; }
        for (int n = 0; n < 9; n++) { ctx->Ah[n] = (double*)q; q += b1; }
        ctx->csnd = (double*)q; q += b1;
        ctx->phi = (double*)q; q += b1;
        ctx->acc = (double*)q; q += 5 * b1;
        if (p->viscous)
            for (int d = 0; d < 3; d++) { ctx->Fv[d] = (double*)q; q += up(nv * 4 * 8); }
        if (fvm) {
            for (int n = 0; n < 12; n++) { ctx->geo[n] = (double*)q; q += b1; }
            ctx->Ufv = (double*)q; q += 5 * b1;
        }
        phi_bytes = b1;
    } else {
        const size_t b1 = up(nc * 4);
        if (!r32) {  // the reference form reads the caller's Float32 Q, metrics and J
            ctx->Q32 = (float*)q; q += 6 * b1;
            // one pack of seven planes per direction, b1 bytes apart: A_d (3), A_d/|A_d| (3),
            // |A_d| — the tensor the TMA sweeps copy a tile of at once
            for (int d = 0; d < 3; d++) {
                for (int n = 0; n < 3; n++) { ctx->m32.A[3 * d + n] = (float*)q; q += b1; }
                for (int n = 0; n < 3; n++) { ctx->m32.H[3 * d + n] = (float*)q; q += b1; }
                ctx->m32.S[d] = (float*)q; q += b1;
            }
            ctx->m32.J = (float*)q; q += b1;
            ctx->acc32b = (float*)q; q += 5 * b1;
        } else {
            for (int n = 0; n < 9; n++) { ctx->m32.H[n] = (float*)q; q += b1; }
            for (int d = 0; d < 3; d++) { ctx->m32.S[d] = (float*)q; q += b1; }
        }
        ctx->phi32 = (float*)q; q += b1;
        ctx->acc32 = (float*)q; q += 5 * b1;
        if (p->viscous)
            for (int d = 0; d < 3; d++) { ctx->Fv32[d] = (float*)q; q += up(nv * 4 * 4); }
        phi_bytes = b1;
    }
    ctx->dscalar = (double*)q;
    ctx->kstat = (unsigned*)(q + 8);
    ctx->tile_ctr = (unsigned*)(q + 16);  // three counters
    // the TMA-staged FP32 sweeps for the mixed form (F3D_NO_TMA=1 selects the direct-load
    // sweeps, for comparison)
    const char* no_tma = std::getenv("F3D_NO_TMA");
    const bool want_tma = p->precision == F3D_PREC_MIXED && !fvm && sweep_tma_usable(ctx->dp) &&
                          !(no_tma && no_tma[0] == '1');
    // phi outside cells 1..Nt-2 is never written; keep it defined (CUDA.zeros in solver.jl:296)
    if ((e = cudaMemset(mx ? (void*)ctx->phi32 : (void*)ctx->phi, 0, phi_bytes)) != cudaSuccess ||
        (e = cudaMemset(q, 0, 32)) != cudaSuccess || (e = sweep_configure()) != cudaSuccess ||
        (fvm && (e = fvm_configure()) != cudaSuccess) || (want_tma && (e = sweep_tma_configure()) != cudaSuccess)) {
        cudaFree(ctx->slab);
        if (ctx->extra) cudaFree(ctx->extra);
        delete ctx;
        std::fprintf(stderr, "f3d_create: %s\n", cudaGetErrorString(e));
        return F3D_ERR_CUDA;
    }
    if (want_tma) {
        ctx->tma_maps = std::aligned_alloc(64, (sweep_maps_bytes() + 63) & ~(size_t)63);
        const float* pack[3] = {ctx->m32.A[0], ctx->m32.A[3], ctx->m32.A[6]};
        ctx->epi_maps = std::aligned_alloc(64, (epi_maps_bytes() + 63) & ~(size_t)63);
        if (ctx->tma_maps && ctx->epi_maps &&
            make_sweep_maps(ctx->dp, ctx->Q32, pack, up(nc * 4), ctx->phi32, ctx->tma_maps) == cudaSuccess) {
            ctx->use_tma = true;
        } else {  // no tensor maps on this driver: the direct-load sweeps
            std::free(ctx->tma_maps);
            std::free(ctx->epi_maps);
            ctx->tma_maps = ctx->epi_maps = nullptr;
        }
    }
    *out = ctx;
    return F3D_OK;
}

int f3d_destroy(f3d_ctx* ctx) {
    if (!ctx) return F3D_OK;
    cudaSetDevice(ctx->device);
    if (ctx->step_graph) cudaGraphExecDestroy(ctx->step_graph);
    if (ctx->adj_slab) cudaFree(ctx->adj_slab);
    if (ctx->lsave) cudaFree(ctx->lsave);
    if (ctx->extra) cudaFree(ctx->extra);
    std::free(ctx->tma_maps);
    std::free(ctx->epi_maps);
    cudaError_t e = cudaFree(ctx->slab);
    delete ctx;
    return e == cudaSuccess ? F3D_OK : F3D_ERR_CUDA;
}

const char* f3d_last_error(const f3d_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int f3d_scratch_bytes(const f3d_ctx* ctx, size_t* bytes) {
    if (!ctx || !bytes) return F3D_ERR_ARG;
    *bytes = ctx->slab_bytes;
    return F3D_OK;
}

int f3d_set_metrics(f3d_ctx* ctx, const double* const metrics[9], const double* jac, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!metrics) return fail(ctx, F3D_ERR_ARG, "null metrics array");
    if ((rc = check_ptrs(ctx, {metrics[0], metrics[1], metrics[2], metrics[3], metrics[4], metrics[5], metrics[6],
                              metrics[7], metrics[8], jac})))
        return rc;
    for (int n = 0; n < 9; n++) ctx->m[n] = metrics[n];
    ctx->J = jac;
    drop_step_graph(ctx);  // a captured step holds the previous metric pointers
    if (mixed(ctx)) {
        MetricPtrs mp;
        for (int n = 0; n < 9; n++) mp.m[n] = metrics[n];
        mp.J = jac;
        F3D_CUDA(ctx, launch_metric_prep32(ctx->dp, mp, ctx->m32, (cudaStream_t)stream));
    } else {
        F3D_CUDA(ctx, launch_metric_prep(ctx->dp, ctx->m, ctx->S, ctx->Ah, (cudaStream_t)stream));
    }
    ctx->metrics_set = true;
    return F3D_OK;
}

int f3d_compute_metrics(f3d_ctx* ctx, const double* x, const double* y, const double* z, double* const metrics[9],
                        double* jac, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!metrics) return fail(ctx, F3D_ERR_ARG, "null metrics array");
    if ((rc = check_ptrs(ctx, {x, y, z, metrics[0], metrics[1], metrics[2], metrics[3], metrics[4], metrics[5],
                              metrics[6], metrics[7], metrics[8], jac})))
        return rc;
    F3D_CUDA(ctx, launch_metrics(ctx->dp, x, y, z, metrics, jac, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_c2prim(f3d_ctx* ctx, const double* U, double* Q, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Q}))) return rc;
    F3D_CUDA(ctx, launch_c2prim_interior(ctx->dp, U, Q, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_prim2c(f3d_ctx* ctx, const double* Q, double* U, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Q}))) return rc;
    F3D_CUDA(ctx, launch_prim2c(ctx->dp, Q, U, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_lincomb(f3d_ctx* ctx, double* U, const double* Un, double a, double b, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Un}))) return rc;
    F3D_CUDA(ctx, launch_lincomb(ctx->dp, U, Un, a, b, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_fill_ghosts(f3d_ctx* ctx, double* Q, double* U, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    for (int f = 0; f < 6 && !rc; f++)
        if (ctx->params.bc[f].kind == F3D_BC_INFLOW_PROFILE && !ctx->dp.prof[f])
            rc = fail(ctx, F3D_ERR_STATE, "inflow profile not set (call f3d_set_inflow_profile)");
    if (rc || (rc = check_ptrs(ctx, {U, Q}))) return rc;
    F3D_CUDA(ctx, launch_prim_fill(ctx->dp, U, Q, U, nullptr, 1, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_rhs(f3d_ctx* ctx, const double* Q, double* dUdt, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q, dUdt}))) return rc;
    SweepArgs last;
    std::memset(&last, 0, sizeof(last));
    last.out_mode = OUT_RHS;
    last.out = dUdt;
    return run_rhs(ctx, Q, dUdt, last, (cudaStream_t)stream);
}

int f3d_rk3_stage(f3d_ctx* ctx, int stage, double dt, double* U, double* Un, double* Q, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Un, Q}))) return rc;
    if (stage < 1 || stage > 3) return fail(ctx, F3D_ERR_ARG, "stage must be 1, 2 or 3");
    return run_stage(ctx, stage, dt, U, Un, Q, (cudaStream_t)stream);
}

int f3d_rk3_steps(f3d_ctx* ctx, int nsteps, double dt, double* U, double* Un, double* Q, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Un, Q}))) return rc;
    if (nsteps < 0) return fail(ctx, F3D_ERR_ARG, "nsteps must be >= 0");
    cudaStream_t st = (cudaStream_t)stream;
    // Q's FP32 copy (mixed precision) or the sound speed (FP64) is made once here; afterwards
    // every stage's primitive fill rewrites it, so the stages inside the step (and the graph)
    // skip it. The filter between steps changes U only, not Q.
    const bool mx = mixed(ctx);
    if (nsteps > 0) {
        if (mx) F3D_CUDA(ctx, launch_to_f32(Q, ctx->Q32, 6 * ctx->dp.plane, st));
        else if (ctx->params.scheme == F3D_SCHEME_FDM) F3D_CUDA(ctx, launch_sound(ctx->dp, Q, ctx->csnd, st));
    }
    const int filt = ctx->params.filter, every = ctx->params.filter_interval;
    auto after_step = [&]() {  // solver.jl:446-470: filter after every `every`-th step
        ctx->tt++;
        return (filt && ctx->tt % every == 0) ? apply_filter(ctx, U, Un, Q, st) : F3D_OK;
    };
    if (st == nullptr) {  // the legacy stream cannot be captured: plain launches
        for (int t = 0; t < nsteps; t++) {
            for (int s = 1; s <= 3; s++)
                if ((rc = run_stage(ctx, s, dt, U, Un, Q, st, true))) return rc;
            if ((rc = after_step())) return rc;
        }
        return F3D_OK;
    }
    const void* key[4] = {U, Un, Q, st};
    bool hit = ctx->step_graph && ctx->g_dt == dt;
    for (int n = 0; n < 4 && hit; n++) hit = ctx->g_key[n] == key[n];
    if (!hit) {
        if (ctx->step_graph) {
            cudaGraphExecDestroy(ctx->step_graph);
            ctx->step_graph = nullptr;
        }
        cudaGraph_t g;
        F3D_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int src = F3D_OK;
        for (int s = 1; s <= 3 && !src; s++) src = run_stage(ctx, s, dt, U, Un, Q, st, true);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (src) return src;
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&ctx->step_graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaGraphInstantiate");
        for (int n = 0; n < 4; n++) ctx->g_key[n] = key[n];
        ctx->g_dt = dt;
    }
    for (int t = 0; t < nsteps; t++) {
        F3D_CUDA(ctx, cudaGraphLaunch(ctx->step_graph, st));
        if ((rc = after_step())) return rc;
    }
    return F3D_OK;
}

int f3d_rk3_step(f3d_ctx* ctx, double dt, double* U, double* Un, double* Q, f3d_stream stream) {
    return f3d_rk3_steps(ctx, 1, dt, U, Un, Q, stream);
}

// ---- F3D_PREC_REF32 entries (Float32 arrays) ---------------------------------------------
int f3d_set_metrics_f32(f3d_ctx* ctx, const float* const metrics[9], const float* jac, f3d_stream stream) {
    int rc = check_ctx32(ctx, false);
    if (rc) return rc;
    if (!metrics) return fail(ctx, F3D_ERR_ARG, "null metrics array");
    if ((rc = check_ptrs(ctx, {metrics[0], metrics[1], metrics[2], metrics[3], metrics[4], metrics[5], metrics[6],
                              metrics[7], metrics[8], jac})))
        return rc;
    for (int n = 0; n < 9; n++) ctx->m32.A[n] = const_cast<float*>(metrics[n]);  // read only
    ctx->m32.J = const_cast<float*>(jac);
    drop_step_graph(ctx);
    F3D_CUDA(ctx, launch_metric_prep_ref32(ctx->dp, ctx->m32, (cudaStream_t)stream));
    ctx->metrics_set = true;
    return F3D_OK;
}

int f3d_compute_metrics_f32(f3d_ctx* ctx, const float* x, const float* y, const float* z, float* const metrics[9],
                            float* jac, int coefficients, f3d_stream stream) {
    int rc = check_ctx32(ctx, false);
    if (rc) return rc;
    if (!metrics) return fail(ctx, F3D_ERR_ARG, "null metrics array");
    if (coefficients != F3D_METRICS_READFORT && coefficients != F3D_METRICS_PARSE_MESH)
        return fail(ctx, F3D_ERR_ARG, "coefficients must be F3D_METRICS_READFORT or F3D_METRICS_PARSE_MESH");
    if ((rc = check_ptrs(ctx, {x, y, z, metrics[0], metrics[1], metrics[2], metrics[3], metrics[4], metrics[5],
                              metrics[6], metrics[7], metrics[8], jac})))
        return rc;
    F3D_CUDA(ctx, launch_metrics32(ctx->dp, x, y, z, metrics, jac, coefficients == F3D_METRICS_PARSE_MESH,
                                   (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_c2prim_f32(f3d_ctx* ctx, const float* U, float* Q, f3d_stream stream) {
    int rc = check_ctx32(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Q}))) return rc;
    F3D_CUDA(ctx, launch_prim_fill32(ctx->dp, U, Q, nullptr, 2, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_prim2c_f32(f3d_ctx* ctx, const float* Q, float* U, f3d_stream stream) {
    int rc = check_ctx32(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Q}))) return rc;
    F3D_CUDA(ctx, launch_prim2c32(ctx->dp, Q, U, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_fill_ghosts_f32(f3d_ctx* ctx, float* Q, float* U, f3d_stream stream) {
    int rc = check_ctx32(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Q}))) return rc;
    F3D_CUDA(ctx, launch_prim_fill32(ctx->dp, U, Q, U, 1, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_rhs_f32(f3d_ctx* ctx, const float* Q, float* dUdt, f3d_stream stream) {
    int rc = check_ctx32(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q, dUdt}))) return rc;
    SweepArgs last;
    std::memset(&last, 0, sizeof(last));
    last.out_mode = OUT_RHS;
    last.out32 = dUdt;
    return run_rhs32(ctx, Q, last, (cudaStream_t)stream);
}

int f3d_rk3_stage_f32(f3d_ctx* ctx, int stage, float dt, float* U, float* Un, float* Q, f3d_stream stream) {
    int rc = check_ctx32(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Un, Q}))) return rc;
    if (stage < 1 || stage > 3) return fail(ctx, F3D_ERR_ARG, "stage must be 1, 2 or 3");
    return run_stage32(ctx, stage, dt, U, Un, Q, (cudaStream_t)stream);
}

int f3d_rk3_steps_f32(f3d_ctx* ctx, int nsteps, float dt, float* U, float* Un, float* Q, f3d_stream stream) {
    int rc = check_ctx32(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Un, Q}))) return rc;
    if (nsteps < 0) return fail(ctx, F3D_ERR_ARG, "nsteps must be >= 0");
    cudaStream_t st = (cudaStream_t)stream;
    if (st == nullptr) {  // the legacy stream cannot be captured
        for (int t = 0; t < nsteps; t++)
            for (int s = 1; s <= 3; s++)
                if ((rc = run_stage32(ctx, s, dt, U, Un, Q, st))) return rc;
        return F3D_OK;
    }
    const void* key[4] = {U, Un, Q, st};
    bool hit = ctx->step_graph && ctx->g_dt == (double)dt;
    for (int n = 0; n < 4 && hit; n++) hit = ctx->g_key[n] == key[n];
    if (!hit) {
        drop_step_graph(ctx);
        cudaGraph_t g;
        F3D_CUDA(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int src = F3D_OK;
        for (int s = 1; s <= 3 && !src; s++) src = run_stage32(ctx, s, dt, U, Un, Q, st);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (src) return src;
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaStreamEndCapture");
        ce = cudaGraphInstantiate(&ctx->step_graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaGraphInstantiate");
        for (int n = 0; n < 4; n++) ctx->g_key[n] = key[n];
        ctx->g_dt = (double)dt;
    }
    for (int t = 0; t < nsteps; t++) F3D_CUDA(ctx, cudaGraphLaunch(ctx->step_graph, st));
    return F3D_OK;
}

int f3d_debug_round_f32(const double* in, float* out, long long n, f3d_stream stream) {
    if (!in || !out || n < 0) return F3D_ERR_ARG;
    if (((uintptr_t)in & 15u) || ((uintptr_t)out & 7u)) return F3D_ERR_ALIGN;
    return launch_to_f32(in, out, n, (cudaStream_t)stream) == cudaSuccess ? F3D_OK : F3D_ERR_CUDA;
}

int f3d_filter(f3d_ctx* ctx, double* U, double* Un, const double* Q, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U, Un, Q}))) return rc;
    if (!ctx->params.filter) return fail(ctx, F3D_ERR_ARG, "params.filter is F3D_FILTER_NONE");
    return apply_filter(ctx, U, Un, Q, (cudaStream_t)stream);
}

int f3d_local_dt(f3d_ctx* ctx, const double* Q, double* dt, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q, dt}))) return rc;
    F3D_CUDA(ctx, launch_local_dt(ctx->dp, Q, ctx->m, ctx->J,
                                  ctx->params.lts_cfl > 0.0 ? ctx->params.lts_cfl : 0.5, dt, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_set_coordinates(f3d_ctx* ctx, const double* x, const double* y, const double* z, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {x, y, z}))) return rc;
    if (ctx->params.scheme == F3D_SCHEME_FDM) return F3D_OK;
    F3D_CUDA(ctx, launch_face_geometry(ctx->dp, x, y, z, ctx->geo, (cudaStream_t)stream));
    ctx->coords_set = true;
    drop_step_graph(ctx);
    return F3D_OK;
}

int f3d_set_metrics_cotangent(f3d_ctx* ctx, double* const metrics_bar[9], double* jac_bar, f3d_stream stream) {
    (void)stream;
    int rc = check_ctx(ctx, false);
    if (rc) return rc;
    if (!metrics_bar) {
        for (int n = 0; n < 9; n++) ctx->mbar[n] = nullptr;
        ctx->Jbar = nullptr;
        return F3D_OK;
    }
    if ((rc = adjoint_supported(ctx))) return rc;
    if ((rc = check_ptrs(ctx, {metrics_bar[0], metrics_bar[1], metrics_bar[2], metrics_bar[3], metrics_bar[4],
                              metrics_bar[5], metrics_bar[6], metrics_bar[7], metrics_bar[8], jac_bar})))
        return rc;
    if (!ctx->lsave) {
        cudaError_t e = cudaMalloc(&ctx->lsave, (size_t)ctx->dp.plane * 10 * sizeof(double));
        if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMalloc (forward RHS of the stage states)");
    }
    for (int n = 0; n < 9; n++) ctx->mbar[n] = metrics_bar[n];
    ctx->Jbar = jac_bar;
    return F3D_OK;
}

int f3d_set_inflow_profile_cotangent(f3d_ctx* ctx, int face, double* prof_bar, f3d_stream stream) {
    (void)stream;
    if (!ctx) return F3D_ERR_ARG;
    if (face < 0 || face > 5) return fail(ctx, F3D_ERR_ARG, "face must be 0..5");
    if (ctx->params.bc[face].kind != F3D_BC_INFLOW_PROFILE)
        return fail(ctx, F3D_ERR_ARG, "face is not an F3D_BC_INFLOW_PROFILE face");
    if (prof_bar) {
        int rc = check_ptrs(ctx, {prof_bar});
        if (rc) return rc;
    }
    ctx->dp.profb[face] = prof_bar;
    return F3D_OK;
}

int f3d_set_inflow_profile(f3d_ctx* ctx, int face, const double* prof, f3d_stream stream) {
    (void)stream;
    if (!ctx) return F3D_ERR_ARG;
    if (face < 0 || face > 5) return fail(ctx, F3D_ERR_ARG, "face must be 0..5");
    if (ctx->params.bc[face].kind != F3D_BC_INFLOW_PROFILE)
        return fail(ctx, F3D_ERR_ARG, "face is not an F3D_BC_INFLOW_PROFILE face");
    int rc = check_ptrs(ctx, {prof});
    if (rc) return rc;
    ctx->dp.prof[face] = prof;
    drop_step_graph(ctx);
    return F3D_OK;
}

int f3d_rhs_vjp(f3d_ctx* ctx, const double* U, const double* Lbar, double* Ubar, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Lbar, Ubar}))) return rc;
    if ((rc = adjoint_supported(ctx)) || (rc = adjoint_alloc(ctx))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    F3D_CUDA(ctx, cudaMemsetAsync(Ubar, 0, (size_t)ctx->dp.plane * 5 * sizeof(double), st));
    if ((rc = prep_state(ctx, U, ctx->Qst[0], ctx->cst_[0], ctx->phst[0], st))) return rc;
    const bool mbar = ctx->mbar[0] != nullptr;
    if (mbar && (rc = rhs_prepared(ctx, ctx->Qst[0], ctx->cst_[0], ctx->phst[0], ctx->Lt, st))) return rc;
    return rhs_vjp_prepared(ctx, U, ctx->Qst[0], ctx->cst_[0], ctx->phst[0], Lbar, Ubar, 1.0, 0.0, st,
                            mbar ? ctx->Lt : nullptr);
}

// SSP-RK3 step U1 = U0 + dt L(U0), U2 = 3/4 U0 + 1/4 (U1 + dt L(U1)),
// U3 = 1/3 U0 + 2/3 (U2 + dt L(U2)), with L(U) = RHS(ghost-filled c2Prim(U)); the stage
// states are recomputed from U0, then the stages are reversed.
int f3d_rk3_step_vjp(f3d_ctx* ctx, double dt, const double* U0, const double* Ubar_next, double* Ubar,
                     f3d_stream stream) {
    return f3d_rk3_step_vjp_stages(ctx, dt, U0, Ubar_next, Ubar, nullptr, nullptr, stream);
}

// The same, also returning the three stage states V_s (U0, U1, U2) and the cotangents of
// their RHS values L(V_s) (dt times the stage cotangents the step VJP applies).
int f3d_rk3_step_vjp_stages(f3d_ctx* ctx, double dt, const double* U0, const double* Ubar_next, double* Ubar,
                            double* Ustage, double* Lbar_stage, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U0, Ubar_next, Ubar}))) return rc;
    if (Ubar == Ubar_next || Ubar == U0) return fail(ctx, F3D_ERR_ARG, "Ubar must not alias U0 or Ubar_next");
    for (double* o : {Ustage, Lbar_stage})
        if (o && (rc = check_ptrs(ctx, {o}))) return rc;
    if ((rc = adjoint_supported(ctx)) || (rc = adjoint_alloc(ctx))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const DevParams& P = ctx->dp;
    // forward recompute of the two intermediate stage states U1, U2
    const double* Us[3] = {U0, ctx->U1, ctx->U2};
    const bool mbar = ctx->mbar[0] != nullptr;
    const size_t lbytes = (size_t)P.plane * 5 * sizeof(double);
    if ((rc = prep_state(ctx, U0, ctx->Qst[0], ctx->cst_[0], ctx->phst[0], st))) return rc;
    if ((rc = rhs_prepared(ctx, ctx->Qst[0], ctx->cst_[0], ctx->phst[0], ctx->Lt, st))) return rc;
    if (mbar) F3D_CUDA(ctx, cudaMemcpyAsync(ctx->lsave, ctx->Lt, lbytes, cudaMemcpyDeviceToDevice, st));
    F3D_CUDA(ctx, launch_axpby(P, ctx->U1, U0, 1.0, ctx->Lt, dt, st));
    if ((rc = prep_state(ctx, ctx->U1, ctx->Qst[1], ctx->cst_[1], ctx->phst[1], st))) return rc;
    if ((rc = rhs_prepared(ctx, ctx->Qst[1], ctx->cst_[1], ctx->phst[1], ctx->Lt, st))) return rc;
    if (mbar)
        F3D_CUDA(ctx, cudaMemcpyAsync(ctx->lsave + 5 * P.plane, ctx->Lt, lbytes, cudaMemcpyDeviceToDevice, st));
    F3D_CUDA(ctx, launch_axpby(P, ctx->U2, ctx->U1, 0.25, ctx->Lt, 0.25 * dt, st));
    F3D_CUDA(ctx, launch_axpby(P, ctx->U2, ctx->U2, 1.0, U0, 0.75, st));
    // each stage's VJP needs its prepared state (Q, sound speed, sensor): kept from the
    // recompute, or, with adjoint_lean (one shared cache), prepared again (c2Prim with the
    // ghost fill, and the sensor) for stages 1 and 0
    const bool lean = ctx->params.adjoint_lean != 0;
    if ((rc = prep_state(ctx, ctx->U2, ctx->Qst[2], ctx->cst_[2], ctx->phst[2], st))) return rc;
    // the metric cotangents' Jacobian term needs L(U2) too (one more RHS)
    if (mbar && (rc = rhs_prepared(ctx, ctx->Qst[2], ctx->cst_[2], ctx->phst[2], ctx->Lt, st))) return rc;
    const double* Lf[3] = {ctx->lsave, ctx->lsave ? ctx->lsave + 5 * P.plane : nullptr, ctx->Lt};
    const long long pl5 = 5 * P.plane;
    if (Ustage)
        for (int k = 0; k < 3; k++) F3D_CUDA(ctx, launch_axpby(P, Ustage + k * pl5, Us[k], 1.0, nullptr, 0.0, st));
    auto vjp = [&](int k, const double* Lb, double* out) {
        if (Lbar_stage) F3D_CUDA(ctx, launch_axpby(P, Lbar_stage + k * pl5, Lb, dt, nullptr, 0.0, st));
        int r = (lean && k < 2) ? prep_state(ctx, Us[k], ctx->Qst[k], ctx->cst_[k], ctx->phst[k], st) : 0;
        return r ? r : rhs_vjp_prepared(ctx, Us[k], ctx->Qst[k], ctx->cst_[k], ctx->phst[k], Lb, out, dt, 1.0, st,
                                        mbar ? Lf[k] : nullptr);
    };
    // stage 3: U3 = 1/3 U0 + 2/3 W, W = U2 + dt L(U2)
    F3D_CUDA(ctx, launch_axpby(P, Ubar, Ubar_next, 1.0 / 3.0, nullptr, 0.0, st));
    F3D_CUDA(ctx, launch_axpby(P, ctx->Xb, Ubar_next, 2.0 / 3.0, nullptr, 0.0, st));  // Wb
    F3D_CUDA(ctx, launch_axpby(P, ctx->Yb, ctx->Xb, 1.0, nullptr, 0.0, st));          // U2b = Wb + dt J^T Wb
    if ((rc = vjp(2, ctx->Xb, ctx->Yb))) return rc;
    // stage 2: U2 = 3/4 U0 + 1/4 V, V = U1 + dt L(U1)
    F3D_CUDA(ctx, launch_axpby(P, Ubar, Ubar, 1.0, ctx->Yb, 0.75, st));
    F3D_CUDA(ctx, launch_axpby(P, ctx->Xb, ctx->Yb, 0.25, nullptr, 0.0, st));  // Vb
    F3D_CUDA(ctx, launch_axpby(P, ctx->Yb, ctx->Xb, 1.0, nullptr, 0.0, st));    // U1b = Vb + dt J^T Vb
    if ((rc = vjp(1, ctx->Xb, ctx->Yb))) return rc;
    // stage 1: U1 = U0 + dt L(U0)
    F3D_CUDA(ctx, launch_axpby(P, Ubar, Ubar, 1.0, ctx->Yb, 1.0, st));
    return vjp(0, ctx->Yb, Ubar);
}

int f3d_kernel_count(void) { return K_NKIND; }

const char* f3d_kernel_name(int kind) { return (kind >= 0 && kind < K_NKIND) ? kKernelNames[kind] : "unknown"; }

int f3d_profile_step(f3d_ctx* ctx, double dt, double* U, double* Un, double* Q, f3d_stream stream, double* ms_out,
                     int* launches_out) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Un, Q}))) return rc;
    if (!ms_out || !launches_out) return fail(ctx, F3D_ERR_ARG, "null output arrays");
    cudaStream_t st = (cudaStream_t)stream;
    Prof prof;
    for (int i = 0; i < Prof::kMax; i++) F3D_CUDA(ctx, cudaEventCreate(&prof.ev[i]));
    ctx->prof = &prof;
    mark(ctx, -1, st);
    // as inside f3d_rk3_steps, the mixed form's FP32 copy of Q and the FP64 sound speed are
    // made for the first stage only: every stage's primitive fill rewrites them
    for (int s = 1; s <= 3 && !rc; s++) rc = run_stage(ctx, s, dt, U, Un, Q, st, s > 1);
    ctx->prof = nullptr;
    cudaError_t e = cudaStreamSynchronize(st);
    for (int k = 0; k < K_NKIND; k++) {
        ms_out[k] = 0.0;
        launches_out[k] = 0;
    }
    if (!rc && e == cudaSuccess) {
        for (int i = 1; i < prof.n; i++) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, prof.ev[i - 1], prof.ev[i]);
            ms_out[prof.kind[i]] += ms;
            launches_out[prof.kind[i]] += prof.nl[i];
        }
    }
    for (int i = 0; i < Prof::kMax; i++) cudaEventDestroy(prof.ev[i]);
    if (rc) return rc;
    return e == cudaSuccess ? F3D_OK : cuda_fail(ctx, e, "cudaStreamSynchronize");
}

int f3d_cfl_dt(f3d_ctx* ctx, const double* Q, double cfl, double* dt_out, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q}))) return rc;
    if (!dt_out || !(cfl > 0.0)) return fail(ctx, F3D_ERR_ARG, "need cfl > 0 and dt_out");
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned long long inf = 0x7ff0000000000000ULL;
    F3D_CUDA(ctx, cudaMemcpyAsync(ctx->dscalar, &inf, 8, cudaMemcpyHostToDevice, st));
    F3D_CUDA(ctx, launch_cfl(ctx->dp, Q, ctx->m, ctx->J, cfl, (unsigned long long*)ctx->dscalar, st));
    F3D_CUDA(ctx, cudaMemcpyAsync(dt_out, ctx->dscalar, 8, cudaMemcpyDeviceToHost, st));
    F3D_CUDA(ctx, cudaStreamSynchronize(st));
    return F3D_OK;
}

int f3d_check_finite(f3d_ctx* ctx, const double* U, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {U}))) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int flag[2] = {0, 0};  // the non-finite flag, then the kernel status word
    F3D_CUDA(ctx, cudaMemsetAsync(ctx->dscalar, 0, 8, st));
    F3D_CUDA(ctx, launch_check_finite(ctx->dp, U, (int*)ctx->dscalar, st));
    F3D_CUDA(ctx, cudaMemcpyAsync(&flag[0], ctx->dscalar, 4, cudaMemcpyDeviceToHost, st));
    F3D_CUDA(ctx, cudaMemcpyAsync(&flag[1], ctx->kstat, 4, cudaMemcpyDeviceToHost, st));
    F3D_CUDA(ctx, cudaStreamSynchronize(st));
    if (flag[1]) return fail(ctx, F3D_ERR_CUDA, "a sweep's tile copy did not complete (kernel status word set)");
    return flag[0] ? fail(ctx, F3D_ERR_NONFINITE, "non-finite value in U") : F3D_OK;
}

int f3d_debug_sensor(f3d_ctx* ctx, const double* Q, double* phi, f3d_stream stream) {
    int rc = check_ctx(ctx, false);
    if (rc || (rc = check_ptrs(ctx, {Q, phi}))) return rc;
    F3D_CUDA(ctx, launch_sensor(ctx->dp, Q, phi, (cudaStream_t)stream, true));
    return F3D_OK;
}

int f3d_debug_split(f3d_ctx* ctx, int dir, const double* Q, double* Fp, double* Fm, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q, Fp, Fm}))) return rc;
    if (dir < 0 || dir > 2) return fail(ctx, F3D_ERR_ARG, "dir must be 0, 1 or 2");
    if (mixed(ctx)) return fail(ctx, F3D_ERR_UNSUPPORTED, "stage intermediates are FP64-only");
    cudaStream_t st = (cudaStream_t)stream;
    F3D_CUDA(ctx, launch_sound(ctx->dp, Q, ctx->csnd, st));
    const double* A[3] = {ctx->m[3 * dir], ctx->m[3 * dir + 1], ctx->m[3 * dir + 2]};
    const double* H[3] = {ctx->Ah[3 * dir], ctx->Ah[3 * dir + 1], ctx->Ah[3 * dir + 2]};
    F3D_CUDA(ctx, launch_split_debug(ctx->dp, Q, ctx->csnd, A, H, ctx->S[dir], Fp, Fm, st));
    return F3D_OK;
}

int f3d_debug_face_flux(f3d_ctx* ctx, int dir, const double* Q, const double* phi, double* F, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q, F}))) return rc;
    if (dir < 0 || dir > 2) return fail(ctx, F3D_ERR_ARG, "dir must be 0, 1 or 2");
    const bool hybrid = ctx->dp.fixed_branch < 0;
    if (hybrid && !phi) return fail(ctx, F3D_ERR_ARG, "hybrid thresholds need phi");
    if (mixed(ctx)) return fail(ctx, F3D_ERR_UNSUPPORTED, "stage intermediates are FP64-only");
    cudaStream_t st = (cudaStream_t)stream;
    if (ctx->params.scheme != F3D_SCHEME_FDM) {  // FVM.jl face fluxes from U = prim2c(Q)
        F3D_CUDA(ctx, launch_prim2c(ctx->dp, Q, ctx->Ufv, st));
        SweepArgs a = sweep_args(ctx, dir, Q, hybrid, phi);
        a.out_mode = OUT_FACES;
        a.faces = F;
        a.Fv = nullptr;
        F3D_CUDA(ctx, launch_fvm_sweep(dir, ctx->params.scheme == F3D_SCHEME_FVM_EIGEN, a, ctx->Ufv, ctx->geo, st));
        return F3D_OK;
    }
    F3D_CUDA(ctx, launch_sound(ctx->dp, Q, ctx->csnd, st));
    SweepArgs a = sweep_args(ctx, dir, Q, hybrid, phi);
    a.out_mode = OUT_FACES;
    a.faces = F;
    a.Fv = nullptr;
    F3D_CUDA(ctx, launch_sweep(dir, a, st));
    return F3D_OK;
}

int f3d_debug_viscous(f3d_ctx* ctx, const double* Q, double* Fvx, double* Fvy, double* Fvz, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {Q, Fvx, Fvy, Fvz}))) return rc;
    if (mixed(ctx)) return fail(ctx, F3D_ERR_UNSUPPORTED, "stage intermediates are FP64-only");
    F3D_CUDA(ctx, launch_viscous(ctx->dp, Q, ctx->m, ctx->J, Fvx, Fvy, Fvz, (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_div(f3d_ctx* ctx, double* U, const double* Fx, const double* Fy, const double* Fz, const double* Fvx,
            const double* Fvy, const double* Fvz, double dt, f3d_stream stream) {
    int rc = check_ctx(ctx, true);
    if (rc || (rc = check_ptrs(ctx, {U, Fx, Fy, Fz}))) return rc;
    const bool visc = Fvx || Fvy || Fvz;
    if (visc && (rc = check_ptrs(ctx, {Fvx, Fvy, Fvz}))) return rc;
    F3D_CUDA(ctx, launch_div_ref(ctx->dp, U, Fx, Fy, Fz, visc ? Fvx : nullptr, Fvy, Fvz, ctx->J, dt,
                                 (cudaStream_t)stream));
    return F3D_OK;
}

int f3d_measure_pipes(double* fp64_tflops, double* fp32_tflops) {
    if (!fp64_tflops || !fp32_tflops) return F3D_ERR_ARG;
    return measure_pipes(fp64_tflops, fp32_tflops) == cudaSuccess ? F3D_OK : F3D_ERR_CUDA;
}

}  // extern "C"
