// k_ref32.cu — pointwise kernels of the F3D_PREC_REF32 form: the reference's own Float32
// arithmetic on Float32 arrays (its U, Un, Q, metrics and J are Float32 CuArrays).
//   k_metric_prep_ref32  |A_d| and A_d / |A_d| per cell in Float32 (split.jl:17-24 forms
//                        them per call from the Float32 metrics; here once per metric set);
//   k_prim_interior32    c2Prim at interior cells (utils.jl:2-30, clamps at eps(Float32));
//   k_prim_ghost32       the composed ghost rules (boundary.jl:1-156, mpi.jl periodic
//                        semantics) from the interior result;
//   k_prim2c32           prim2c over every cell (utils.jl:33-54).
// The operations are written with round-to-nearest intrinsics in the reference's order,
// so no multiply-add is contracted and the results are bitwise those of the Float32
// restatement of the same formulas.
#include "f3d_kernels.cuh"

namespace f3d {

namespace {
constexpr int R32_THREADS = 256;
unsigned r32_blocks(long long n) { return (unsigned)((n + R32_THREADS - 1) / R32_THREADS); }

// Julia's max / min: NaN in either argument is returned
__device__ __forceinline__ float jmax32(float a, float b) { return a != a ? a : (b != b ? b : (a < b ? b : a)); }

__device__ __forceinline__ float kin32(float rho, float u, float v, float w) {
    return __fmul_rn(__fmul_rn(0.5f, rho), __fadd_rn(__fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)), __fmul_rn(w, w)));
}

__device__ __forceinline__ void c2prim32(const DevParams& P, const float U[5], float q[6]) {
    const float rho = jmax32(U[0], P.eps32);
    const float rinv = __fdiv_rn(1.0f, rho);
    const float u = __fmul_rn(U[1], rinv), v = __fmul_rn(U[2], rinv), w = __fmul_rn(U[3], rinv);
    const float ei = jmax32(__fsub_rn(U[4], kin32(rho, u, v, w)), P.eps32);
    const float p = __fmul_rn(P.gm1_32, ei);
    q[0] = rho; q[1] = u; q[2] = v; q[3] = w; q[4] = p;
    q[5] = __fdiv_rn(p, __fmul_rn(rho, P.rg32));
}

__device__ __forceinline__ void prim2c32(const DevParams& P, const float q[6], float U[5]) {
    U[0] = q[0];
    U[1] = __fmul_rn(q[1], q[0]);
    U[2] = __fmul_rn(q[2], q[0]);
    U[3] = __fmul_rn(q[3], q[0]);
    U[4] = __fadd_rn(__fdiv_rn(q[4], P.gm1_32), kin32(q[0], q[1], q[2], q[3]));
}

// the chain's transforms in Float32 (apply_chain in FP64): Dirichlet state, mirrors, and
// the isothermal rule T = 2 T_w - T, rho = p / (Rg T)
__device__ __forceinline__ void apply_chain32(const DevParams& P, const GhostChain& c, float q[6]) {
    if (c.dirichlet >= 0) {
        const BcDev& b = P.bc[c.dirichlet];
        q[0] = (float)b.rho; q[1] = (float)b.u; q[2] = (float)b.v; q[3] = (float)b.w; q[4] = (float)b.p;
        q[5] = __fdiv_rn(q[4], __fmul_rn(q[0], P.rg32));
    }
    if (c.nmirror & 1) {
        q[1] = -q[1];
        q[2] = -q[2];
        q[3] = -q[3];
    }
    if (c.iso_face >= 0) {
        q[5] = __fsub_rn(__fmul_rn(2.0f, (float)P.bc[c.iso_face].t_wall), q[5]);
        q[0] = __fdiv_rn(q[4], __fmul_rn(P.rg32, q[5]));
    }
}
}  // namespace

__global__ void k_metric_prep_ref32(const DevParams P, MetricPtrs32 m) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const float a = m.A[3 * d][c], b = m.A[3 * d + 1][c], e = m.A[3 * d + 2][c];
        const float s = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b)), __fmul_rn(e, e)));
        const float si = __fdiv_rn(1.0f, s);
        m.S[d][c] = s;
        m.H[3 * d][c] = __fmul_rn(a, si);
        m.H[3 * d + 1][c] = __fmul_rn(b, si);
        m.H[3 * d + 2][c] = __fmul_rn(e, si);
    }
}

__global__ void k_prim_interior32(const DevParams P, const float* U, float* Q) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.nx * P.ny * P.nz) return;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    const long long c = lin3(P, i + NG, j + NG, k + NG), pl = P.plane;
    float u[5], q[6];
#pragma unroll
    for (int n = 0; n < 5; n++) u[n] = U[c + n * pl];
    c2prim32(P, u, q);
#pragma unroll
    for (int n = 0; n < 6; n++) Q[c + n * pl] = q[n];
}

__global__ void k_prim_ghost32(const DevParams P, const float* U, float* Q, float* Ug) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    if (i >= NG && i < P.nx + NG && j >= NG && j < P.ny + NG && k >= NG && k < P.nz + NG) return;
    const long long pl = P.plane;
    const GhostChain ch = resolve_ghost(P, i, j, k);
    const long long s = lin3(P, ch.si, ch.sj, ch.sk);
    float q[6];
    if (ch.dirichlet < 0) {
#pragma unroll
        for (int n = 0; n < 6; n++) q[n] = Q[s + n * pl];
    }
    apply_chain32(P, ch, q);
#pragma unroll
    for (int n = 0; n < 6; n++) Q[c + n * pl] = q[n];
    if (Ug) {
        if (ch.nontrivial) {
            float u[5];
            prim2c32(P, q, u);
#pragma unroll
            for (int n = 0; n < 5; n++) Ug[c + n * pl] = u[n];
        } else {
#pragma unroll
            for (int n = 0; n < 5; n++) Ug[c + n * pl] = U[s + n * pl];
        }
    }
}

__global__ void k_prim2c32(const DevParams P, const float* Q, float* U) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    float q[6], u[5];
#pragma unroll
    for (int n = 0; n < 6; n++) q[n] = Q[c + n * P.plane];
    prim2c32(P, q, u);
#pragma unroll
    for (int n = 0; n < 5; n++) U[c + n * P.plane] = u[n];
}

cudaError_t launch_metric_prep_ref32(const DevParams& P, const MetricPtrs32& m, cudaStream_t st) {
    k_metric_prep_ref32<<<r32_blocks(P.plane), R32_THREADS, 0, st>>>(P, m);
    return cudaGetLastError();
}

// mode 0: c2Prim at interior cells, then the ghost rules; 1: the ghost rules only (Q's
// interior given, fillGhost); 2: c2Prim at interior cells only
cudaError_t launch_prim_fill32(const DevParams& P, const float* U, float* Q, float* Ug, int mode, cudaStream_t st) {
    if (mode != 1)
        k_prim_interior32<<<r32_blocks((long long)P.nx * P.ny * P.nz), R32_THREADS, 0, st>>>(P, U, Q);
    if (mode != 2) k_prim_ghost32<<<r32_blocks(P.plane), R32_THREADS, 0, st>>>(P, U, Q, Ug);
    return cudaGetLastError();
}

cudaError_t launch_prim2c32(const DevParams& P, const float* Q, float* U, cudaStream_t st) {
    k_prim2c32<<<r32_blocks(P.plane), R32_THREADS, 0, st>>>(P, Q, U);
    return cudaGetLastError();
}

}  // namespace f3d
