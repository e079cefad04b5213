// f3d_kernels.cuh — launch interfaces between the C-ABI layer (api.cu) and the kernels.
#pragma once
#include <string>

#include "f3d_common.cuh"
#include "f3d_flux.cuh"

namespace f3d {

enum OutMode { OUT_SET = 0, OUT_ADD = 1, OUT_RHS = 2, OUT_STAGE = 3, OUT_FACES = 4 };

// Arguments of one sweep. The field pointers are typed by the sweep's arithmetic: double
// arrays for the FP64 form, float arrays (FP32 copies) for the mixed form (fp32 = 1).
// J, U, Un, out and faces are double in both forms.
struct SweepArgs {
    DevParams P;
    const void* Q;        // primitive state (Nt^3 x 6), ghost-filled
    const void* csnd;     // FP64 form: sound speed per cell for the split
    const void* A[3];     // metric row of the sweep direction (J^-1 scaled)
    const void* Ah[3];    // A * (1/|A|)
    const void* S;        // |A|
    const void* phi;      // shock sensor (only read when P.fixed_branch < 0)
    const void* Fv;       // viscous flux of this direction ((Nt-4)^3 x 4) or null
    const double* J;      // Jacobian
    void* acc;            // RHS accumulator (U layout)
    const float* acc2;    // mixed form, last sweep: the eta sweep's own differences (FP32);
                          // the three directions are then summed in FP64 (null otherwise)
    double* out;          // OUT_RHS destination (may alias acc in the FP64 form)
    double* U;            // OUT_STAGE state, updated in place
    double* Un;           // OUT_STAGE stage-start copy
    double* faces;        // OUT_FACES destination (Fx/Fy/Fz shape) or null
    double dt, ca, cb;    // OUT_STAGE: U = ca*(U + dt J acc) + cb*Un when combine
    const double* dtl;    // OUT_STAGE with local time stepping: per-cell dt replacing dt
    int out_mode;
    int combine;
    int stage1_copy;      // OUT_STAGE of stage 1: Un = U before the update
    int fp32;             // 1: the mixed-precision (FP32) sweep
    // F3D_PREC_REF32 (the FP32 sweep on the caller's Float32 arrays): Float32 outputs
    const float* J32;     // Jacobian
    float* out32;         // OUT_RHS destination
    float* U32;           // OUT_STAGE state
    float* Un32;          // OUT_STAGE stage-start copy
    float dt32, ca32, cb32;
    unsigned* kstat;      // kernel status word of the context (bit 0: a TMA tile wait gave up)
    unsigned* tile_ctr;   // TMA sweeps: next-tile counters of the three directions (zeroed per RHS)
};

// Metric and Jacobian cotangents accumulated by the viscous VJP (null m[0]: none)
struct MetricBar {
    double* m[9];
    double* J;
    double scale;
};

// Arguments of one sweep VJP (k_adjoint.cu, FP64, component-wise reconstruction)
struct AdjArgs {
    DevParams P;
    const double* Q;      // forward primitive state, ghost-filled
    const double* csnd;   // forward split sound speed
    const double* A[3];
    const double* Ah[3];
    const double* S;
    const double* phi;    // forward sensor (hybrid)
    const double* J;
    const double* Lb;     // cotangent of the RHS (U layout, interior cells)
    double* Qb;           // accumulated cotangent of Q (6 x Nt^3)
    double* mb[3];        // optional: accumulated cotangent of this direction's metric row
    double mscale;        //   (scaled by mscale, the VJP's alpha)
};

cudaError_t adjoint_configure();
cudaError_t launch_sweep_vjp(int dir, const AdjArgs& a, cudaStream_t st);
cudaError_t launch_viscous_vjp(const DevParams& P, const double* Q, const double* const m[9], const double* J,
                               const double* Lb, double* Fvb[3], double* gb, double* Qb, cudaStream_t st,
                               double* const mbar[9] = nullptr, double* Jbar = nullptr, double mscale = 0.0);
// Jbar += mscale sum_n Lb L / J at interior cells: the RHS's direct dependence on J (L = J D)
cudaError_t launch_jbar(const DevParams& P, const double* Lb, const double* L, const double* J, double* Jbar,
                        double mscale, cudaStream_t st);
cudaError_t launch_fill_vjp(const DevParams& P, const double* Q, double* Qb, double pscale, cudaStream_t st);
cudaError_t launch_c2prim_vjp(const DevParams& P, const double* U, const double* Qb, double* out, double alpha,
                              double beta, cudaStream_t st);
cudaError_t launch_axpby(const DevParams& P, double* out, const double* x, double a, const double* y, double b,
                         cudaStream_t st);

// parameter validation and device constants (api.cu)
int validate_params(const f3d_params& p, std::string& why);
DevParams make_dev_params(const f3d_params& p);

cudaError_t sweep_configure();
cudaError_t launch_sweep(int dir, const SweepArgs& a, cudaStream_t st);
// TMA-staged FP32 sweeps of the mixed form (k_sweep_tma.cu): usable when the x extent with
// ghosts is a multiple of 4; maps3 holds the three directions' tensor maps
bool sweep_tma_usable(const DevParams& P);
cudaError_t sweep_tma_configure();
size_t sweep_maps_bytes();
cudaError_t make_sweep_maps(const DevParams& P, const float* q32, const float* const pack[3], size_t pack_stride,
                            const float* phi, void* maps3);
// epi: the last sweep's staged Phase C maps (make_epi_maps) or null (direct loads)
cudaError_t launch_sweep_tma(int dir, const SweepArgs& a, const void* maps3, const void* epi, cudaStream_t st);
size_t epi_maps_bytes();
cudaError_t make_epi_maps(const DevParams& P, const float* acc, const float* acc2, const double* J,
                          const double* U, const double* Un, void* out);

// finite-volume scheme (k_fvm.cu): geo = (nx, ny, nz, area) of the faces of x, y, z at
// their left cells; U the conserved state the faces reconstruct from
cudaError_t fvm_configure();
cudaError_t launch_face_geometry(const DevParams& P, const double* x, const double* y, const double* z,
                                 double* const geo[12], cudaStream_t st);
cudaError_t launch_fvm_sweep(int dir, bool eigen, const SweepArgs& a, const double* U, const double* const geo[12],
                             cudaStream_t st);
cudaError_t launch_stage_update(const DevParams& P, const double* acc, const double* J, double dt, double* U,
                                double* Un, int stage1_copy, int combine, double ca, double cb, cudaStream_t st,
                                const double* dtl = nullptr);

// step components beside the stage (k_step_extras.cu): local time step of every interior
// cell (utils.jl:73-99) and the explicit filters of U (utils.jl:102-315)
cudaError_t launch_local_dt(const DevParams& P, const double* Q, const double* const m[9], const double* J,
                            double lts_cfl, double* dt, cudaStream_t st);
cudaError_t launch_filter_dir(const DevParams& P, int dir, int mode, double s0, double rth, const double* Q,
                              double* U, const double* Un, double* sc, cudaStream_t st);

// metric pointer bundles (passed by value to kernels)
struct MetricPtrs {
    const double* m[9];
    const double* J;
};
struct MetricPtrs32 {
    float* A[9];
    float* H[9];
    float* S[3];
    float* J;
};

// pointwise / stencil kernels (k_pointwise.cu)
// Q at every cell from the interior of U (c2Prim) or of Q itself (from_q), with the
// ghost layers produced by the composed boundary rules. U ghosts are written when
// U_ghost_out is not null. csnd (optional) receives the split's sound speed.
// F3D_PREC_REF32 pointwise kernels (k_ref32.cu)
cudaError_t launch_metric_prep_ref32(const DevParams& P, const MetricPtrs32& m, cudaStream_t st);
cudaError_t launch_prim_fill32(const DevParams& P, const float* U, float* Q, float* Ug, int mode, cudaStream_t st);
cudaError_t launch_prim2c32(const DevParams& P, const float* Q, float* U, cudaStream_t st);
cudaError_t launch_prim_fill(const DevParams& P, const double* U, double* Q, double* U_ghost_out, double* csnd,
                             int from_q, cudaStream_t st, float* Q32 = nullptr);
cudaError_t launch_to_f32(const double* src, float* dst, long long n, cudaStream_t st);
cudaError_t launch_sensor32(const DevParams& P, const float* Q32, float* phi, cudaStream_t st);
cudaError_t launch_metric_prep32(const DevParams& P, const MetricPtrs& m, const MetricPtrs32& o, cudaStream_t st);
cudaError_t launch_c2prim_interior(const DevParams& P, const double* U, double* Q, cudaStream_t st);
cudaError_t launch_prim2c(const DevParams& P, const double* Q, double* U, cudaStream_t st);
cudaError_t launch_lincomb(const DevParams& P, double* U, const double* Un, double a, double b, cudaStream_t st);
cudaError_t launch_sound(const DevParams& P, const double* Q, double* csnd, cudaStream_t st);
// exact: phi bit for bit as the oracle's; otherwise values that give the same branch map
// (FP32 away from the thresholds, FP64 near them)
cudaError_t launch_sensor(const DevParams& P, const double* Q, double* phi, cudaStream_t st, bool exact = false);
cudaError_t launch_metric_prep(const DevParams& P, const double* const m[9], double* S[3], double* Ah[9],
                               cudaStream_t st);
cudaError_t launch_split_debug(const DevParams& P, const double* Q, const double* csnd, const double* const A[3],
                               const double* const Ah[3], const double* S, double* Fp, double* Fm, cudaStream_t st);
cudaError_t launch_div_ref(const DevParams& P, double* U, const double* Fx, const double* Fy, const double* Fz,
                           const double* Fvx, const double* Fvy, const double* Fvz, const double* J, double dt,
                           cudaStream_t st);
cudaError_t launch_check_finite(const DevParams& P, const double* U, int* flag, cudaStream_t st);
cudaError_t launch_cfl(const DevParams& P, const double* Q, const double* const m[9], const double* J, double cfl,
                       unsigned long long* dtbits, cudaStream_t st);

// viscous fluxes (k_viscous.cu): FP64 from the FP64 arrays, or FP32 from the FP32 copies
cudaError_t launch_viscous(const DevParams& P, const double* Q, const double* const m[9], const double* J,
                           double* Fvx, double* Fvy, double* Fvz, cudaStream_t st);
cudaError_t launch_viscous32(const DevParams& P, const float* Q, const float* const m[9], const float* J,
                             float* Fvx, float* Fvy, float* Fvz, cudaStream_t st);

// metrics from coordinates (k_metrics.cu)
// nine metric outputs and J of the Float32 set-up metrics (k_metrics32)
struct MetricOut32 {
    float* m[9];
    float* J;
};
cudaError_t launch_metrics32(const DevParams& P, const float* x, const float* y, const float* z,
                             float* const m[9], float* J, bool f64coef, cudaStream_t st);
cudaError_t launch_metrics(const DevParams& P, const double* x, const double* y, const double* z,
                           double* const m[9], double* J, cudaStream_t st);

// pipe throughput probe (k_pointwise.cu)
cudaError_t measure_pipes(double* fp64_tflops, double* fp32_tflops);

}  // namespace f3d
