/*
 * flame3d_gpu.h — C ABI of libflame3d_gpu.so, the GB300 (sm_103a) finite-difference
 * right-hand side and SSP-RK3 stage of the Flame3D compressible Navier–Stokes solver.
 *
 * The library replaces the @cuda launch sites of the reference's finite-difference
 * path: flowAdvance (solver.jl:19-189, finite_volume=false branch at solver.jl:133-188),
 * the RK3 stage loop (solver.jl:416-444), exchange_ghost (mpi.jl:2-103) and fillGhost
 * (boundary.jl:151-156). A Julia driver binds it with ccall; every array keeps the
 * reference layout: Julia column-major (Nx+2NG, Ny+2NG, Nz+2NG, nvar), i fastest, so the
 * 0-based linear index of (i,j,k,n) is i + Nxt*(j + Nyt*(k + Nzt*n)).
 *
 * Conventions
 *  - All array arguments are DEVICE pointers owned by the caller (Julia CuArrays or torch
 *    tensors). The library never frees them. Scratch space is allocated in f3d_create and
 *    released in f3d_destroy.
 *  - Every entry point returns an int status (F3D_OK = 0). No exception or abort crosses
 *    the ABI. f3d_last_error(ctx) returns a message for the last failure on that ctx.
 *  - Calls are asynchronous on the given stream (NULL = legacy default stream). A context is
 *    not thread-safe: use one context per host thread / stream.
 *  - Physical state (U, Un, Q, metrics, J, x/y/z) is always double precision. The
 *    precision field of f3d_params selects the arithmetic of the flux kernels.
 */
#ifndef FLAME3D_GPU_H
#define FLAME3D_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define F3D_VERSION 10000 /* 1.0.0 */

/* status codes */
#define F3D_OK 0
#define F3D_ERR_ARG 1          /* invalid argument (null pointer, bad dims, bad enum)   */
#define F3D_ERR_ALIGN 2        /* a pointer is not 16-byte aligned                      */
#define F3D_ERR_CUDA 3         /* a CUDA runtime call or a host allocation failed       */
#define F3D_ERR_NONFINITE 4    /* a NaN/Inf was found in the checked state              */
#define F3D_ERR_UNSUPPORTED 5  /* valid request that the library does not implement      */
#define F3D_ERR_STATE 6        /* call order violated (e.g. metrics not set)            */
#define F3D_ERR_TOO_LARGE 7    /* the grid needs more scratch than f3d_rhs_noalloc holds */

/* flux-vector splitting (run.jl:69 splitMethod; split.jl) */
#define F3D_SPLIT_SW 0   /* Steger–Warming, split.jl:2-68   */
#define F3D_SPLIT_LF 1   /* local Lax–Friedrichs, split.jl:70-108 */
#define F3D_SPLIT_VL 2   /* van Leer, split.jl:110-183      */
#define F3D_SPLIT_AUSM 3 /* AUSM, split.jl:185-255          */

/* right-hand-side family (run.jl:64-65 finite_volume / eigen_reconstruction) */
#define F3D_SCHEME_FDM 0       /* flux splitting + hybrid reconstruction of the split fluxes
                                  (split.jl, schemes.jl): the finite-difference path       */
#define F3D_SCHEME_FVM_EIGEN 1 /* finite volume: Roe-averaged characteristic reconstruction
                                  of U + HLLC (FVM.jl Eigen_reconstruct_*, HLLC_Flux)      */
#define F3D_SCHEME_FVM_CONS 2  /* finite volume: component-wise reconstruction of U + HLLC
                                  (FVM.jl Conser_reconstruct_*)                            */

/* arithmetic of the flux kernels */
#define F3D_PREC_FP64 0  /* everything in FP64: the drop-in, parity at 1e-12             */
#define F3D_PREC_MIXED 1 /* FP32 split/reconstruction/weights/viscous; FP64 state, EOS,
                            metrics/J, RK accumulation and reductions                   */
#define F3D_PREC_REF32 2 /* the reference's own arithmetic on its Float32 arrays: U, Un, Q,
                            metrics and J are Float32 and every step is Float32 except the
                            WENO7 weights (FP64, schemes.jl:178-185); the *_f32 entries
                            below, the FP64-array entries refuse such a context          */

/* explicit filters of U (utils.jl:102-315) */
#define F3D_FILTER_NONE 0
#define F3D_FILTER_LINEAR 1     /* 8th-order linear filter, linearFilter_x/y/z              */
#define F3D_FILTER_NONLINEAR 2  /* shock-capturing filter: pressure sensor pre_x/y/z, then
                                   the 4-point dissipative filter filter_x/y/z               */

/* sub-grid models (viscous.jl:66-106) */
#define F3D_LES_NONE 0
#define F3D_LES_SMAGORINSKY 1   /* C_s = 0.1, Pr_t = 0.9                                     */
#define F3D_LES_WALE 2          /* C_w = 0.325, Pr_t = 0.9                                   */

/* ghost-cell rules, one per face (x-, x+, y-, y+, z-, z+). Faces are filled in the
 * order x, y, z over the full transverse extent including ghosts, which is the
 * order of fill_x, fill_y, fill_z in boundary.jl:151-156. */
#define F3D_BC_PERIODIC 0        /* copy from the opposite side, mpi.jl:2-103 with self as neighbour */
#define F3D_BC_DIRICHLET 1       /* fixed (rho,u,v,w,p); T = p/(rho Rg), boundary.jl:12-38,98-118   */
#define F3D_BC_ZERO_GRADIENT 2   /* copy the adjacent interior layer, boundary.jl:42-51             */
#define F3D_BC_WALL_ADIABATIC 3  /* mirror: rho,p,T even, u,v,w odd, boundary.jl:67-93             */
#define F3D_BC_WALL_ISOTHERMAL 4 /* mirror u,v,w odd, p even, T = 2 T_wall - T_in, rho = p/(Rg T)  */
#define F3D_BC_INFLOW_PROFILE 5  /* Dirichlet with (rho,u,v,w,p) per boundary point from a caller
                                    array (f3d_set_inflow_profile); T = p/(rho Rg). The inlet
                                    rule of boundary.jl:10-38 with a per-point state, as fed by an
                                    inflow file (SCU-benchmark/flow-inlet.dat)                 */

typedef struct f3d_bc {
    int32_t kind;
    int32_t pad_;
    double rho, u, v, w, p; /* F3D_BC_DIRICHLET state                        */
    double t_wall;          /* F3D_BC_WALL_ISOTHERMAL wall temperature         */
} f3d_bc;

typedef struct f3d_params {
    int32_t nx, ny, nz;  /* interior cells per direction (Nxp, Nyp, Nzp; run.jl:84-86),    */
                         /* each >= 4 = NG (a periodic fill copies NG interior layers;   */
                         /* smaller grids: F3D_ERR_ARG); a quasi-2D case uses 4 layers  */
    int32_t ng;          /* ghost layers; must be 4 (parse_mesh.jl:6)                    */
    double gamma;        /* run.jl:8                                                     */
    double rg;           /* run.jl:9                                                     */
    double cp;           /* run.jl:10; 0 means Rg*gamma/(gamma-1)                        */
    double c_s, t_s;     /* Sutherland constants, run.jl:11-12                           */
    double pr;           /* Prandtl number, run.jl:13                                    */
    double phi1, phi2, phi3; /* hybrid thresholds, run.jl:70-72                          */
    double linear_phi;   /* UP7/CD6 blend of the linear scheme, run.jl:73-77             */
    double clamp_eps;    /* lower clamp of rho and e_int in c2Prim (utils.jl:12,18);
                            0 means the reference value eps(Float32) = 2^-23              */
    int32_t split_method;   /* F3D_SPLIT_*                                               */
    int32_t character;      /* 1: characteristic-wise (advect_xc), 0: component-wise     */
    int32_t viscous;        /* 1: add viscous and heat fluxes (viscous.jl)               */
    int32_t precision;      /* F3D_PREC_*                                                */
    f3d_bc bc[6];           /* x-, x+, y-, y+, z-, z+                                    */
    int32_t scheme;         /* F3D_SCHEME_*; the finite-volume schemes are FP64 only       */
    int32_t adjoint_lean;   /* 1: the step VJP keeps one prepared stage state instead of three
                               (16 grid-sized arrays less, two more preparations per step) */
    /* step components beside the RK stage (run.jl:3-5, 21-22, 49-54; off by default)      */
    int32_t lts;            /* 1: local time stepping: each stage advances every cell by its
                               own dt = lts_cfl min_d(V/S_d/(u_d+c)) (utils.jl:73-99,
                               div.jl:52-101); the dt argument of the stage entries is unused */
    int32_t filter;         /* F3D_FILTER_*: applied to U after every filter_interval-th step
                               of f3d_rk3_steps (solver.jl:446-470), or by f3d_filter          */
    int32_t filter_interval;
    int32_t les;            /* F3D_LES_*: eddy viscosity in the viscous fluxes (viscous.jl:66-106) */
    double lts_cfl;         /* run.jl:22                                                   */
    double filter_s0;       /* filter strength, run.jl:54                                  */
    double filter_rth;      /* shock-capturing filter threshold, run.jl:53                 */
} f3d_params;

typedef struct f3d_ctx f3d_ctx;
typedef struct CUstream_st* f3d_stream; /* a cudaStream_t */

/* ---- lifetime ------------------------------------------------------------------ */

/* Library version, F3D_VERSION. */
int f3d_version(void);

/* Fill *p with the reference's run.jl defaults (FDM path, SW split, characteristic,
 * viscous, thresholds 0.05/1/10, the boundary.jl inlet/outlet/wall/farfield/periodic
 * BCs) for an nx x ny x nz interior grid. Replaces the compile-time consts of run.jl:3-77. */
int f3d_default_params(int nx, int ny, int nz, f3d_params* p);

/* Validate p, allocate the device scratch for this grid and return a context.
 * Replaces the allocations of solver.jl:293-337. */
int f3d_create(const f3d_params* p, f3d_ctx** out);
int f3d_destroy(f3d_ctx* ctx);
const char* f3d_last_error(const f3d_ctx* ctx);

/* Bytes of device scratch the context holds. */
int f3d_scratch_bytes(const f3d_ctx* ctx, size_t* bytes);

/* ---- geometry ------------------------------------------------------------------ */

/* Borrow the nine J^-1-scaled metric arrays (dxi/dx, dxi/dy, dxi/dz, deta/dx, ...,
 * dzeta/dz, the order of metrics.h5, parse_mesh.jl:240-248) and J, each (Nxt,Nyt,Nzt),
 * and derive |grad xi_d| (solver.jl:286-288). The pointers must stay valid while the
 * context uses them. Replaces the metric load of solver.jl:238-288. */
int f3d_set_metrics(f3d_ctx* ctx, const double* const metrics[9], const double* jac,
                    f3d_stream stream);

/* Cell-centre coordinates (Nxt,Nyt,Nzt each, ghost layers filled as solver.jl:682-829
 * extrapolates them) for the finite-volume schemes: the unit normal and area of every face
 * (FVM.jl:16-29) are computed once here, in FP64, and kept in the context. Required before
 * any call that needs the metrics when params.scheme is a finite-volume scheme (else
 * F3D_ERR_STATE); a no-op for F3D_SCHEME_FDM. The arrays are read only by the work this
 * call queues on the stream. */
int f3d_set_coordinates(f3d_ctx* ctx, const double* x, const double* y, const double* z, f3d_stream stream);

/* Compute metrics and J from coordinates x,y,z (Nxt,Nyt,Nzt with ghost coordinates) with
 * the CD6 / one-sided CD2 formulas of parse_mesh.jl:139-248, in FP64 on the device. */
int f3d_compute_metrics(f3d_ctx* ctx, const double* x, const double* y, const double* z,
                        double* const metrics[9], double* jac, f3d_stream stream);

/* ---- pointwise kernels (utils.jl) ----------------------------------------------- */

/* U -> Q (rho,u,v,w,p,T) at interior cells with the clamps of utils.jl:2-30. */
int f3d_c2prim(f3d_ctx* ctx, const double* U, double* Q, f3d_stream stream);
/* Q -> U at every cell, utils.jl:33-54. */
int f3d_prim2c(f3d_ctx* ctx, const double* Q, double* U, f3d_stream stream);
/* U = a U + b Un at interior cells, utils.jl:57-70. */
int f3d_lincomb(f3d_ctx* ctx, double* U, const double* Un, double a, double b,
                f3d_stream stream);
/* Ghost layers of Q (6 vars) and U (5 vars) from their interiors by the context's BCs:
 * exchange_ghost (mpi.jl:2-103) on one GPU followed by fillGhost (boundary.jl:151-156). */
int f3d_fill_ghosts(f3d_ctx* ctx, double* Q, double* U, f3d_stream stream);

/* ---- right-hand side ------------------------------------------------------------ */

/* dUdt = L(U) at interior cells (dUdt has the U layout; ghosts are not written) from a
 * ghost-filled Q: shock sensor, flux splitting and hybrid reconstruction in xi, eta,
 * zeta, viscous fluxes and the flux divergence (div.jl:1-50 without the dt factor).
 * Equals (U_after_div - U_before)/dt of one reference stage. The finite-volume schemes
 * reconstruct the conserved variables; here they take U = prim2c(Q) at every cell (the
 * stage entries use the state U itself). */
int f3d_rhs(f3d_ctx* ctx, const double* Q, double* dUdt, f3d_stream stream);

/* One SSP-RK3 stage (stage = 1,2,3) exactly as solver.jl:416-444: stage 1 copies U to
 * Un; U += dt L(Q); stage 2: U = U/4 + 3Un/4; stage 3: U = 2U/3 + Un/3; then
 * Q = c2Prim(U) and the ghost fill of Q and U. Q must be ghost-filled on entry. With
 * params.lts, stage 1 computes the local time steps from its Q and stages 2 and 3 of the
 * same context use them (compute_dt at KRK == 1 only, solver.jl:418-421). */
int f3d_rk3_stage(f3d_ctx* ctx, int stage, double dt, double* U, double* Un, double* Q,
                  f3d_stream stream);

/* nsteps full SSP-RK3 steps (3 stages each). Replays a CUDA graph of one step after the
 * first call with the same pointers. */
int f3d_rk3_steps(f3d_ctx* ctx, int nsteps, double dt, double* U, double* Un, double* Q,
                  f3d_stream stream);
/* One SSP-RK3 step: f3d_rk3_steps with nsteps = 1 (one pass of the loop body of
 * solver.jl:409-470). */
int f3d_rk3_step(f3d_ctx* ctx, double dt, double* U, double* Un, double* Q, f3d_stream stream);

/* Largest stable dt for the given CFL number over interior cells:
 * min over cells and directions of cfl / (J (|U_d| + c |grad xi_d|)), U_d = grad xi_d . u.
 * Synchronises the stream. */
int f3d_cfl_dt(f3d_ctx* ctx, const double* Q, double cfl, double* dt_out,
               f3d_stream stream);

/* Scan the interior of U for NaN/Inf (the reference's NaN check, solver.jl:481-486).
 * Returns F3D_ERR_NONFINITE if one is found. Synchronises the stream. */
int f3d_check_finite(f3d_ctx* ctx, const double* U, f3d_stream stream);

/* ---- right-hand side without device allocation -------------------------------------- */

/* Scratch held by f3d_rhs_noalloc: a file-scope device array of this many bytes, kept by
 * every GPU that loads the library until the process exits. */
#define F3D_NOALLOC_SCRATCH_BYTES (32 * 1024 * 1024)

/* The same dUdt as f3d_create + f3d_set_metrics + f3d_rhs, for callers that cannot
 * allocate device memory: a host whose memory pool has reserved the device's memory and
 * forbids foreign cudaMalloc/cudaFree (a framework allocator, or a job held to a fixed
 * device-memory quota), or a time-critical loop that cannot afford cudaFree's implicit
 * synchronisation of the whole device. No context is needed: p, the nine metrics, J, the
 * ghost-filled Q and dUdt are the caller's; nothing is allocated and no allocating library
 * routine is called. Scratch (|A|, A/|A|, sound speed, sensor and, when viscous, the
 * viscous fluxes: 14 (Nx+8)(Ny+8)(Nz+8) doubles + 12 (Nx+4)(Ny+4)(Nz+4) doubles) lives in
 * one shared device array of F3D_NOALLOC_SCRATCH_BYTES; larger grids return
 * F3D_ERR_TOO_LARGE (about 58^3 interior cells inviscid, 48^3 viscous). The first call on
 * a device looks up that array's device address (cudaGetSymbolAddress, with that device
 * current) and sets kernel attributes for that device; the address is kept for the rest of
 * the process, so a cudaDeviceReset of that device leaves the entry point unusable. Make the
 * first call before any stream capture. Every call uses the same array and leaves its
 * contents behind, so calls whose kernels overlap on the GPU (on different streams or host
 * threads) race: serialise them. Returns F3D_* codes; messages go to stderr.
 * This entry point has no counterpart in the reference, whose kernels take preallocated
 * CuArrays (solver.jl:293-337). */
int f3d_rhs_noalloc(const f3d_params* p, const double* const metrics[9], const double* jac,
                    const double* Q, double* dUdt, f3d_stream stream);

/* One pass of the explicit filter of params.filter over U (interior cells), the three
 * directions in turn, each from a copy Un of U made just before it (solver.jl:447-470);
 * Q supplies the shock-capturing filter's pressure sensor and is not updated (as in the
 * reference). f3d_rk3_steps applies it by itself after every filter_interval-th step. */
int f3d_filter(f3d_ctx* ctx, double* U, double* Un, const double* Q, f3d_stream stream);

/* Local time step of every interior cell (compute_dt, utils.jl:73-99) into dt (U-cell
 * layout, ghosts untouched), with params.lts_cfl (0.5 when unset). */
int f3d_local_dt(f3d_ctx* ctx, const double* Q, double* dt, f3d_stream stream);

/* Borrow the state of an F3D_BC_INFLOW_PROFILE face (0..5 = x-, x+, y-, y+, z-, z+): a
 * device array of 5 x Ta x Tb doubles, variable-major (rho, u, v, w, p), each plane indexed
 * a + Ta * b over the full transverse extent including ghosts: (a, b) = (j, k) with
 * Ta = Ny+8 on x faces, (i, k) with Ta = Nx+8 on y faces, (i, j) with Ta = Nx+8 on z faces.
 * Every ghost layer of the face takes the state of its transverse point. While a face of
 * that kind has no profile, f3d_fill_ghosts and every call that needs the metrics return
 * F3D_ERR_STATE. The caller keeps the array alive and may rewrite it between calls (the
 * kernels read it at each launch). */
int f3d_set_inflow_profile(f3d_ctx* ctx, int face, const double* prof, f3d_stream stream);

/* The rounding of FP64 values to FP32 the mixed form uses for its FP32 copies (integer
 * operations on the IEEE 754 layouts, round to nearest even), on n device values; for
 * checking it against the conversion instruction. No context; no counterpart in the
 * reference. */
int f3d_debug_round_f32(const double* in, float* out, long long n, f3d_stream stream);

/* ---- F3D_PREC_REF32: the reference's Float32 arrays and arithmetic ---------------------
 * The same calls as f3d_set_metrics, f3d_c2prim, f3d_prim2c, f3d_fill_ghosts, f3d_rhs,
 * f3d_rk3_stage and f3d_rk3_steps on Float32 arrays of the same shapes: the reference's
 * CuArray{Float32} U, Un, Q, metrics and J (solver.jl:238-337) pass unchanged. The
 * computation follows the reference's Float32 operations (c2Prim clamps at eps(Float32),
 * Float32 splitting, sensor, UP7/WENO5 and viscous fluxes (with either LES model),
 * WENO7 weights in FP64, Float32 RK update); FP64 entries and these refuse each other's
 * contexts (F3D_ERR_ARG). No inflow-profile faces, local time stepping, filters, adjoint
 * or finite-volume scheme in this form (F3D_ERR_UNSUPPORTED at f3d_create). */
int f3d_set_metrics_f32(f3d_ctx* ctx, const float* const metrics[9], const float* jac, f3d_stream stream);
/* The Float32 metrics and J the reference's set-up writes to metrics.h5, from Float32
 * coordinates with ghosts (Nxt,Nyt,Nzt): the CD6 / one-sided CD2 differences with Float32
 * coefficients (F3D_METRICS_READFORT, SCU-benchmark/readfort.jl:103-181) or with Float64
 * coefficients on Float32 differences, rounded to Float32 (F3D_METRICS_PARSE_MESH,
 * parse_mesh.jl:138-248); every operation rounded to nearest in the Julia loops' order, so
 * the results equal the reference's bit for bit. The outputs can go to f3d_set_metrics_f32. */
#define F3D_METRICS_READFORT 0
#define F3D_METRICS_PARSE_MESH 1
int f3d_compute_metrics_f32(f3d_ctx* ctx, const float* x, const float* y, const float* z,
                            float* const metrics[9], float* jac, int coefficients, f3d_stream stream);
int f3d_c2prim_f32(f3d_ctx* ctx, const float* U, float* Q, f3d_stream stream);
int f3d_prim2c_f32(f3d_ctx* ctx, const float* Q, float* U, f3d_stream stream);
int f3d_fill_ghosts_f32(f3d_ctx* ctx, float* Q, float* U, f3d_stream stream);
int f3d_rhs_f32(f3d_ctx* ctx, const float* Q, float* dUdt, f3d_stream stream);
int f3d_rk3_stage_f32(f3d_ctx* ctx, int stage, float dt, float* U, float* Un, float* Q, f3d_stream stream);
int f3d_rk3_steps_f32(f3d_ctx* ctx, int nsteps, float dt, float* U, float* Un, float* Q, f3d_stream stream);

/* ---- discrete adjoint (FP64, component-wise reconstruction, SW or LF splitting) ---- */

/* Let the adjoint calls of the context also accumulate the cotangent of an inflow-profile
 * face's state (the same 5 x Ta x Tb layout as f3d_set_inflow_profile) into prof_bar: every
 * f3d_rhs_vjp / f3d_rk3_step_vjp adds its share, so after a backward pass prof_bar holds
 * dJ/d(profile) (the caller zeroes it first). nullptr stops the accumulation. No counterpart
 * in the reference. */
int f3d_set_inflow_profile_cotangent(f3d_ctx* ctx, int face, double* prof_bar, f3d_stream stream);

/* Let the adjoint calls also accumulate the cotangents of the nine metrics and of J (the
 * arrays of f3d_set_metrics, same layout; ghost cells included) into metrics_bar / jac_bar:
 * after a backward pass they hold dJ/d(metrics) and dJ/dJ, so a grid parameter's gradient
 * is their dot product with the metrics' derivative in it. The caller zeroes them first;
 * nullptr stops the accumulation. Costs one RHS more per step VJP (the forward RHS of the
 * last stage state, for the J-term) and 10 arrays of scratch. No counterpart in the
 * reference. */
int f3d_set_metrics_cotangent(f3d_ctx* ctx, double* const metrics_bar[9], double* jac_bar, f3d_stream stream);

/* Ubar = (dL/dU)^T Lbar at interior cells (ghost cells of Ubar are zeroed), where
 * L(U) = RHS(ghost-filled c2Prim(U)) is the right-hand side as a function of the interior
 * conserved state. Branches (hybrid scheme choice, minmod, sign splits, c2Prim clamps)
 * are those of the forward state: the exact derivative of the scheme as evaluated.
 * The first adjoint call of a context allocates its adjoint scratch. */
int f3d_rhs_vjp(f3d_ctx* ctx, const double* U, const double* Lbar, double* Ubar, f3d_stream stream);

/* Cotangent of the state at the start of one SSP-RK3 step from the cotangent of the state
 * at its end: Ubar = (dU_{n+1}/dU_n)^T Ubar_next. Recomputes the two intermediate stage
 * states from U0 (2 RHS) and applies three RHS VJPs. Ubar must not alias the inputs.
 * Long trajectories use checkpoints of U every ~sqrt(N) steps and recompute each segment
 * (flame3d_mhd_gb300/adjoint.py). */
int f3d_rk3_step_vjp(f3d_ctx* ctx, double dt, const double* U0, const double* Ubar_next, double* Ubar,
                     f3d_stream stream);

/* f3d_rk3_step_vjp that also writes, when non-null, the step's three stage states
 * V_0 = U0, V_1 = U1, V_2 = U2 into Ustage (3 x 5 planes) and the cotangents of their RHS
 * values L(V_s) into Lbar_stage (3 x 5 planes; dt times the stage cotangent), interior cells
 * (ghost cells zero). With these a caller forms the gradient with respect to any parameter
 * theta of the RHS: the step contributes sum_s <Lbar_s, dL/dtheta at V_s>. */
int f3d_rk3_step_vjp_stages(f3d_ctx* ctx, double dt, const double* U0, const double* Ubar_next, double* Ubar,
                            double* Ustage, double* Lbar_stage, f3d_stream stream);

/* ---- stage-by-stage intermediates in the reference's own array shapes ----------- */

/* phi (Nxt,Nyt,Nzt) at cells 2..Nt-1, schemes.jl:1-24. */
int f3d_debug_sensor(f3d_ctx* ctx, const double* Q, double* phi, f3d_stream stream);
/* Fp, Fm (Nxt,Nyt,Nzt,5) at every cell for direction dir (0=xi,1=eta,2=zeta), split.jl. */
int f3d_debug_split(f3d_ctx* ctx, int dir, const double* Q, double* Fp, double* Fm,
                    f3d_stream stream);
/* Face flux of direction dir in the shape of Fx (Nx+1,Ny,Nz,5), Fy or Fz from Q and phi
 * (advect_x/xc ... advect_z/zc, schemes.jl:86-1643). */
int f3d_debug_face_flux(f3d_ctx* ctx, int dir, const double* Q, const double* phi,
                        double* F, f3d_stream stream);
/* Fv_x, Fv_y, Fv_z ((Nx+2NG-4),(Ny+2NG-4),(Nz+2NG-4),4), viscous.jl:1-133. */
int f3d_debug_viscous(f3d_ctx* ctx, const double* Q, double* Fvx, double* Fvy, double* Fvz,
                      f3d_stream stream);
/* The reference's div kernel (div.jl:1-50) on caller arrays: U += dt J (dF + dFv). */
int f3d_div(f3d_ctx* ctx, double* U, const double* Fx, const double* Fy, const double* Fz,
            const double* Fvx, const double* Fvy, const double* Fvz, double dt,
            f3d_stream stream);

/* ---- profiling and device characterisation ---------------------------------------- */

/* Kernel kinds of one RK3 step: their number and names ("sweep_xi", ...). */
int f3d_kernel_count(void);
const char* f3d_kernel_name(int kind);

/* Run one SSP-RK3 step like f3d_rk3_steps(nsteps=1) without a graph, with a CUDA event
 * after every launch; ms_out[k] / launches_out[k] receive the summed device time and the
 * launch count of kernel kind k (arrays of f3d_kernel_count() entries). Synchronises. */
int f3d_profile_step(f3d_ctx* ctx, double dt, double* U, double* Un, double* Q, f3d_stream stream,
                     double* ms_out, int* launches_out);


/* Measure the FP64 and FP32 FMA pipe throughput of the current device (TFLOP/s) with
 * dependent-FMA chains over every SM, for roofline reporting. Synchronises. */
int f3d_measure_pipes(double* fp64_tflops, double* fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif /* FLAME3D_GPU_H */
