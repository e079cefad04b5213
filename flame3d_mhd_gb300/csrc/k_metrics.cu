// k_metrics.cu — grid metrics and Jacobian from coordinates in FP64 on the device
// (parse_mesh.jl:139-248): sixth-order central differences (CD6) of x, y, z in xi, eta,
// zeta, one-sided second-order differences (CD2) in the three outermost layers of each
// direction, J = 1/det(d(x,y,z)/d(xi,eta,zeta)) and the nine J^-1-scaled metrics (the
// cofactors; parse_mesh.jl:239 "actually after * J^-").
#include "f3d_kernels.cuh"

namespace f3d {

// Set-up code: every product and sum is rounded separately (no FMA contraction), so the
// metrics equal the CPU restatement bitwise.
#define M_ __dmul_rn
#define A_ __dadd_rn
__device__ __forceinline__ double dcoord(const double* f, long long c, long long s, int ii, int Nt) {
    if (ii >= 3 && ii <= Nt - 4)  // CD6, parse_mesh.jl:139-142 (1-based 4..Nt-3)
        return A_(A_(M_(1.0 / 60, A_(f[c + 3 * s], -f[c - 3 * s])), -M_(3.0 / 20, A_(f[c + 2 * s], -f[c - 2 * s]))),
                  M_(3.0 / 4, A_(f[c + s], -f[c - s])));
    if (ii <= 2)  // CD2_L, parse_mesh.jl:144-147
        return A_(A_(M_(2.0, f[c + s]), -M_(0.5, f[c + 2 * s])), -M_(1.5, f[c]));
    return A_(A_(M_(-2.0, f[c - s]), M_(0.5, f[c - 2 * s])), M_(1.5, f[c]));  // CD2_R, parse_mesh.jl:149-152
}

__device__ __forceinline__ double cof(double a, double b, double c, double d) { return A_(M_(a, b), -M_(c, d)); }

__global__ void k_metrics(const DevParams P, const double* x, const double* y, const double* z, double* m0,
                          double* m1, double* m2, double* m3, double* m4, double* m5, double* m6, double* m7,
                          double* m8, double* J) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    const long long sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const double xxi = dcoord(x, c, 1, i, P.nxt), yxi = dcoord(y, c, 1, i, P.nxt), zxi = dcoord(z, c, 1, i, P.nxt);
    const double xet = dcoord(x, c, sy, j, P.nyt), yet = dcoord(y, c, sy, j, P.nyt), zet = dcoord(z, c, sy, j, P.nyt);
    const double xze = dcoord(x, c, sz, k, P.nzt), yze = dcoord(y, c, sz, k, P.nzt), zze = dcoord(z, c, sz, k, P.nzt);
    // parse_mesh.jl:237-248
    const double det = A_(A_(M_(xxi, cof(yet, zze, yze, zet)), -M_(xet, cof(yxi, zze, yze, zxi))),
                          M_(xze, cof(yxi, zet, yet, zxi)));
    J[c] = 1.0 / det;
    m0[c] = cof(yet, zze, yze, zet);
    m1[c] = cof(xze, zet, xet, zze);
    m2[c] = cof(xet, yze, xze, yet);
    m3[c] = cof(yze, zxi, yxi, zze);
    m4[c] = cof(xxi, zze, xze, zxi);
    m5[c] = cof(xze, yxi, xxi, yze);
    m6[c] = cof(yxi, zet, yet, zxi);
    m7[c] = cof(xet, zxi, xxi, zet);
    m8[c] = cof(xxi, yet, xet, yxi);
}
#undef M_
#undef A_

// The reference's Float32 set-up metrics (readfort.jl:103-181 with Float32 coefficients;
// parse_mesh.jl:138-248 with Float64 coefficients on Float32 differences, the sum rounded to
// Float32), every operation rounded to nearest in the Julia loops' order, so the results
// equal the Float32 metrics.h5 the reference writes from the same coordinates.
#define FM __fmul_rn
#define FA __fadd_rn
#define FS __fsub_rn
__device__ __forceinline__ float dcoord32(const float* f, long long c, long long s, int ii, int Nt, bool f64coef) {
    if (ii >= 3 && ii <= Nt - 4) {
        const float d3 = FS(f[c + 3 * s], f[c - 3 * s]), d2 = FS(f[c + 2 * s], f[c - 2 * s]);
        const float d1 = FS(f[c + s], f[c - s]);
        if (f64coef)
            return __double2float_rn(__dadd_rn(__dsub_rn(__dmul_rn(1.0 / 60, (double)d3), __dmul_rn(3.0 / 20, (double)d2)),
                                               __dmul_rn(3.0 / 4, (double)d1)));
        return FA(FS(FM(__fdiv_rn(1.f, 60.f), d3), FM(__fdiv_rn(3.f, 20.f), d2)), FM(__fdiv_rn(3.f, 4.f), d1));
    }
    if (ii <= 2) {  // CD2_L: 2 f[i+1] - 0.5 f[i+2] - 1.5 f[i]
        if (f64coef)
            return __double2float_rn(__dsub_rn(__dsub_rn((double)FM(2.f, f[c + s]), __dmul_rn(0.5, (double)f[c + 2 * s])),
                                               __dmul_rn(1.5, (double)f[c])));
        return FS(FS(FM(2.f, f[c + s]), FM(0.5f, f[c + 2 * s])), FM(1.5f, f[c]));
    }
    // CD2_R: -2 f[i-1] + 0.5 f[i-2] + 1.5 f[i]
    if (f64coef)
        return __double2float_rn(__dadd_rn(__dadd_rn((double)FM(-2.f, f[c - s]), __dmul_rn(0.5, (double)f[c - 2 * s])),
                                           __dmul_rn(1.5, (double)f[c])));
    return FA(FA(FM(-2.f, f[c - s]), FM(0.5f, f[c - 2 * s])), FM(1.5f, f[c]));
}

__device__ __forceinline__ float cof32(float a, float b, float c, float d) { return FS(FM(a, b), FM(c, d)); }

__global__ void k_metrics32(const DevParams P, const float* x, const float* y, const float* z, MetricOut32 m,
                            bool f64coef) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    split3(c, P.dnxt, P.dnyt, i, j, k);
    const long long sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const float xxi = dcoord32(x, c, 1, i, P.nxt, f64coef), yxi = dcoord32(y, c, 1, i, P.nxt, f64coef);
    const float zxi = dcoord32(z, c, 1, i, P.nxt, f64coef);
    const float xet = dcoord32(x, c, sy, j, P.nyt, f64coef), yet = dcoord32(y, c, sy, j, P.nyt, f64coef);
    const float zet = dcoord32(z, c, sy, j, P.nyt, f64coef);
    const float xze = dcoord32(x, c, sz, k, P.nzt, f64coef), yze = dcoord32(y, c, sz, k, P.nzt, f64coef);
    const float zze = dcoord32(z, c, sz, k, P.nzt, f64coef);
    const float det = FA(FS(FM(xxi, cof32(yet, zze, yze, zet)), FM(xet, cof32(yxi, zze, yze, zxi))),
                         FM(xze, cof32(yxi, zet, yet, zxi)));
    m.J[c] = __fdiv_rn(1.f, det);
    m.m[0][c] = cof32(yet, zze, yze, zet);
    m.m[1][c] = cof32(xze, zet, xet, zze);
    m.m[2][c] = cof32(xet, yze, xze, yet);
    m.m[3][c] = cof32(yze, zxi, yxi, zze);
    m.m[4][c] = cof32(xxi, zze, xze, zxi);
    m.m[5][c] = cof32(xze, yxi, xxi, yze);
    m.m[6][c] = cof32(yxi, zet, yet, zxi);
    m.m[7][c] = cof32(xet, zxi, xxi, zet);
    m.m[8][c] = cof32(xxi, yet, xet, yxi);
}
#undef FM
#undef FA
#undef FS

cudaError_t launch_metrics32(const DevParams& P, const float* x, const float* y, const float* z,
                             float* const m[9], float* J, bool f64coef, cudaStream_t st) {
    MetricOut32 o;
    for (int n = 0; n < 9; n++) o.m[n] = m[n];
    o.J = J;
    k_metrics32<<<(unsigned)((P.plane + 255) / 256), 256, 0, st>>>(P, x, y, z, o, f64coef);
    return cudaGetLastError();
}

cudaError_t launch_metrics(const DevParams& P, const double* x, const double* y, const double* z,
                           double* const m[9], double* J, cudaStream_t st) {
    k_metrics<<<(unsigned)((P.plane + 255) / 256), 256, 0, st>>>(P, x, y, z, m[0], m[1], m[2], m[3], m[4], m[5],
                                                                 m[6], m[7], m[8], J);
    return cudaGetLastError();
}

}  // namespace f3d
