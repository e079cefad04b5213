// k_step_extras.cu — step components beside the RK stage, all off by default in the
// reference (run.jl:21-22, 49-54):
//   k_local_dt         local time step of every interior cell (compute_dt, utils.jl:73-99):
//                      lts_cfl * min_d (V / S_d) / (u_d + c) with V = 1/J, S_d = |grad xi_d|
//                      J^-1 and u_d the Cartesian velocity component, as the reference writes it;
//   k_filter_sensor<d> the shock-capturing filter's switch per interior cell (pre_x/y/z,
//                      utils.jl:102-169): r = ((dp0-dp1)^2 + (dp0-dp2)^2) / (2 p^2) + 1e-16
//                      from second differences of p along d, sc = max(0, 1 - rth / r);
//   k_filter<d>        U = Un - s0 (sc_{+1/2} D_{+1/2} - sc_{-1/2} D_{-1/2}) with the
//                      4-point dissipative differences of filter_x/y/z (utils.jl:171-241);
//   k_linear_filter<d> U = Un - s0 (8th-order symmetric difference of Un) (linearFilter_x/y/z,
//                      utils.jl:243-315).
// Each filter direction reads Un, a copy of U made just before it (solver.jl:447-470).
#include "f3d_kernels.cuh"

namespace f3d {

__global__ void k_local_dt(const DevParams P, const double* __restrict__ Q, MetricPtrs m, double cfl, double* dt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)P.nx * P.ny * P.nz;
    if (t >= n) return;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    const long long c = lin3(P, i + NG, j + NG, k + NG), pl = P.plane;
    const double u = Q[c + pl], v = Q[c + 2 * pl], w = Q[c + 3 * pl], T = Q[c + 5 * pl];
    const double V = 1.0 / m.J[c];
    const double cs = sqrt(P.gamma * P.rg * T);
    double S[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double a = m.m[3 * d][c], b = m.m[3 * d + 1][c], e = m.m[3 * d + 2][c];
        S[d] = sqrt(a * a + b * b + e * e);  // s1, s2, s3 of solver.jl:286-288
    }
    const double dtx = V / S[0] / (u + cs), dty = V / S[1] / (v + cs), dtz = V / S[2] / (w + cs);
    dt[c] = fmin(fmin(dtx, dty), dtz) * cfl;
}

cudaError_t launch_local_dt(const DevParams& P, const double* Q, const double* const m[9], const double* J,
                            double lts_cfl, double* dt, cudaStream_t st) {
    MetricPtrs mp;
    for (int a = 0; a < 9; a++) mp.m[a] = m[a];
    mp.J = J;
    const long long n = (long long)P.nx * P.ny * P.nz;
    k_local_dt<<<cdiv(n, 256), 256, 0, st>>>(P, Q, mp, lts_cfl, dt);
    return cudaGetLastError();
}

// interior cell t -> (full linear index, stride along d)
__device__ __forceinline__ bool interior_cell(const DevParams& P, int dir, long long& c, long long& s) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n = (long long)P.nx * P.ny * P.nz;
    if (t >= n) return false;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    c = lin3(P, i + NG, j + NG, k + NG);
    s = dir == 0 ? 1 : (dir == 1 ? (long long)P.nxt : (long long)P.nxt * P.nyt);
    return true;
}

__global__ void k_filter_sensor(const DevParams P, int dir, double rth, const double* __restrict__ Q, double* sc) {
    long long c, s;
    if (!interior_cell(P, dir, c, s)) return;
    const double* p = Q + 4 * P.plane + c;
    const double p1 = p[-2 * s], p2 = p[-s], p3 = p[0], p4 = p[s], p5 = p[2 * s];
    const double d0 = 0.25 * (-p4 + 2.0 * p3 - p2);
    const double d1 = 0.25 * (-p5 + 2.0 * p4 - p3);
    const double d2 = 0.25 * (-p3 + 2.0 * p2 - p1);
    const double r = 0.5 * ((d0 - d1) * (d0 - d1) + (d0 - d2) * (d0 - d2)) / (p3 * p3) + 1e-16;
    const double q = 1.0 - rth / r;
    sc[c] = 0.5 * (q + fabs(q));
}

__global__ void k_filter(const DevParams P, int dir, double s0, const double* __restrict__ sc, double* U,
                         const double* __restrict__ Un) {
    long long c, s;
    if (!interior_cell(P, dir, c, s)) return;
    const double c1 = -0.210383, c2 = 0.039617;
    const double sc1 = 0.5 * (sc[c] + sc[c + s]), sc2 = 0.5 * (sc[c] + sc[c - s]);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const double* f = Un + n * P.plane + c;
        const double dp = c1 * (f[s] - f[0]) + c2 * (f[2 * s] - f[-s]);
        const double dm = c1 * (f[0] - f[-s]) + c2 * (f[s] - f[-2 * s]);
        U[c + n * P.plane] = f[0] - s0 * (sc1 * dp - sc2 * dm);
    }
}

__global__ void k_linear_filter(const DevParams P, int dir, double s0, double* U, const double* __restrict__ Un) {
    long long c, s;
    if (!interior_cell(P, dir, c, s)) return;
    const double d0 = 0.243527493120, d1 = -0.204788880640, d2 = 0.120007591680, d3 = -0.045211119360,
                 d4 = 0.008228661760;
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const double* f = Un + n * P.plane + c;
        U[c + n * P.plane] = f[0] - s0 * (d0 * f[0] + d1 * (f[-s] + f[s]) + d2 * (f[-2 * s] + f[2 * s]) +
                                          d3 * (f[-3 * s] + f[3 * s]) + d4 * (f[-4 * s] + f[4 * s]));
    }
}

cudaError_t launch_filter_dir(const DevParams& P, int dir, int mode, double s0, double rth, const double* Q,
                              double* U, const double* Un, double* sc, cudaStream_t st) {
    const long long n = (long long)P.nx * P.ny * P.nz;
    const unsigned g = cdiv(n, 256);
    if (mode == F3D_FILTER_NONLINEAR) {
        k_filter_sensor<<<g, 256, 0, st>>>(P, dir, rth, Q, sc);
        k_filter<<<g, 256, 0, st>>>(P, dir, s0, sc, U, Un);
    } else {
        k_linear_filter<<<g, 256, 0, st>>>(P, dir, s0, U, Un);
    }
    return cudaGetLastError();
}

}  // namespace f3d
