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

cudaError_t launch_metrics(const DevParams& P, const double* x, const double* y, const double* z,
                           double* const m[9], double* J, cudaStream_t st) {
    k_metrics<<<(unsigned)((P.plane + 255) / 256), 256, 0, st>>>(P, x, y, z, m[0], m[1], m[2], m[3], m[4], m[5],
                                                                 m[6], m[7], m[8], J);
    return cudaGetLastError();
}

}  // namespace f3d
