// k_pointwise.cu — one-thread-per-cell kernels: primitive recovery with the ghost fill,
// the shock sensor, metric preparation, the reference's div kernel, reductions and the
// pipe-throughput probe.
#include "f3d_kernels.cuh"

namespace f3d {

constexpr int PW_THREADS = 256;

static unsigned pw_blocks(long long n) {
    long long b = (n + PW_THREADS - 1) / PW_THREADS;
    return (unsigned)(b < 1 ? 1 : b);
}

__device__ __forceinline__ void cell_ijk(const DevParams& P, long long c, int& i, int& j, int& k) {
    split3(c, P.dnxt, P.dnyt, i, j, k);
}

__device__ __forceinline__ bool is_interior(const DevParams& P, int i, int j, int k) {
    return i >= NG && i < P.nx + NG && j >= NG && j < P.ny + NG && k >= NG && k < P.nz + NG;
}

__device__ __forceinline__ double sound_speed(const DevParams& P, const double q[6]) {
    // split.jl:22 (SW) and split.jl:90,130,205 (LF, VL, AUSM)
    return P.split == F3D_SPLIT_SW ? sqrt(__dmul_rn(P.grg, q[5])) : sqrt(__dmul_rn(P.gamma, q[4]) / q[0]);
}

// c2Prim at interior cells (k_prim_interior), then the composed ghost rules (k_prim_ghost):
// a ghost cell reads the FP64 primitive state its chain starts from, which the first pass
// has just written — bitwise what c2Prim followed by the reference's copies produces —
// instead of recomputing c2Prim there (a quarter of the cells of a 256x64x64 grid are
// ghosts). from_q: Q's interior is given (fillGhost); the first pass then only derives the
// sound speed and the FP32 copy when they are asked for.
__global__ void k_prim_interior(const DevParams P, const double* U, double* Q, double* csnd, float* Q32,
                                int from_q) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)P.nx * P.ny * P.nz) return;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    const long long c = lin3(P, i + NG, j + NG, k + NG), pl = P.plane;
    double q[6];
    if (from_q) {
#pragma unroll
        for (int n = 0; n < 6; n++) q[n] = Q[c + n * pl];
    } else {
        double u[5];
#pragma unroll
        for (int n = 0; n < 5; n++) u[n] = U[c + n * pl];
        if (Q32) c2prim_cell_fast(P, u, q);  // mixed precision
        else c2prim_cell(P, u, q);
#pragma unroll
        for (int n = 0; n < 6; n++) Q[c + n * pl] = q[n];
    }
    if (csnd) csnd[c] = sound_speed(P, q);
    if (Q32) {
#pragma unroll
        for (int n = 0; n < 6; n++) Q32[c + n * pl] = f64_to_f32_rn(q[n]);
    }
}

// Ghost cell number g (0 .. plane - interior - 1) -> (i, j, k): the two z slabs of NG planes
// (every i, j), then the y slabs within the interior z range (every i), then the x slabs of
// the interior (j, k) lines; i runs fastest in the first two, so their accesses coalesce.
__device__ __forceinline__ void ghost_ijk(const DevParams& P, long long g, int& i, int& j, int& k) {
    const long long zs = 2LL * NG * P.nxt * P.nyt;
    const long long ys = 2LL * NG * P.nxt * P.nz;
    if (g < zs) {
        const unsigned q = fdiv((unsigned)g, P.dnxt);
        i = (int)((unsigned)g - q * P.dnxt.d);
        const unsigned kk = fdiv(q, P.dnyt);
        j = (int)(q - kk * P.dnyt.d);
        k = kk < (unsigned)NG ? (int)kk : P.nz + (int)kk;
    } else if (g < zs + ys) {
        const unsigned h = (unsigned)(g - zs);
        const unsigned q = fdiv(h, P.dnxt);
        i = (int)(h - q * P.dnxt.d);
        const unsigned jj = q % (2u * NG), kz = q / (2u * NG);
        j = jj < (unsigned)NG ? (int)jj : P.ny + (int)jj;
        k = (int)kz + NG;
    } else {
        const unsigned h = (unsigned)(g - zs - ys);
        const unsigned ii = h % (2u * NG), q = h / (2u * NG);
        const unsigned kq = fdiv(q, P.dny);
        j = (int)(q - kq * P.dny.d) + NG;
        k = (int)kq + NG;
        i = ii < (unsigned)NG ? (int)ii : P.nx + (int)ii;
    }
}

__global__ void k_prim_ghost(const DevParams P, const double* U, double* Q, double* Ug, double* csnd, float* Q32) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P.plane - (long long)P.nx * P.ny * P.nz) return;
    const long long pl = P.plane;
    int i, j, k;
    ghost_ijk(P, g, i, j, k);
    const long long c = lin3(P, i, j, k);
    double q[6];
    const GhostChain ch = resolve_ghost(P, i, j, k);
    const long long s = lin3(P, ch.si, ch.sj, ch.sk);
    if (ch.dirichlet < 0) {
#pragma unroll
        for (int n = 0; n < 6; n++) q[n] = Q[s + n * pl];
    }
    apply_chain(P, ch, q);
#pragma unroll
    for (int n = 0; n < 6; n++) Q[c + n * pl] = q[n];
    if (Ug) {
        if (ch.nontrivial) {
            double u[5];
            prim2c_cell(P, q, u);
#pragma unroll
            for (int n = 0; n < 5; n++) Ug[c + n * pl] = u[n];
        } else {
#pragma unroll
            for (int n = 0; n < 5; n++) Ug[c + n * pl] = U[s + n * pl];
        }
    }
    if (csnd) csnd[c] = sound_speed(P, q);
    if (Q32) {
#pragma unroll
        for (int n = 0; n < 6; n++) Q32[c + n * pl] = f64_to_f32_rn(q[n]);
    }
}

cudaError_t launch_prim_fill(const DevParams& P, const double* U, double* Q, double* Ug, double* csnd, int from_q,
                             cudaStream_t st, float* Q32) {
    const long long ni = (long long)P.nx * P.ny * P.nz;
    if (!from_q || csnd || Q32) k_prim_interior<<<pw_blocks(ni), PW_THREADS, 0, st>>>(P, U, Q, csnd, Q32, from_q);
    k_prim_ghost<<<pw_blocks(P.plane - ni), PW_THREADS, 0, st>>>(P, U, Q, Ug, csnd, Q32);
    return cudaGetLastError();
}

// FP32 copy of an FP64 array (n elements): the mixed form's view of Q.
__global__ void k_to_f32(const double* __restrict__ src, float* __restrict__ dst, long long n) {
    long long i = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * 2;
    if (i + 1 < n) {
        const double2 v = *reinterpret_cast<const double2*>(src + i);
        *reinterpret_cast<float2*>(dst + i) = make_float2(f64_to_f32_rn(v.x), f64_to_f32_rn(v.y));
    } else if (i < n) {
        dst[i] = f64_to_f32_rn(src[i]);
    }
}
cudaError_t launch_to_f32(const double* src, float* dst, long long n, cudaStream_t st) {
    const long long pairs = (n + 1) / 2;
    k_to_f32<<<pw_blocks(pairs), PW_THREADS, 0, st>>>(src, dst, n);
    return cudaGetLastError();
}

// Shock sensor of the mixed form: the same formula (schemes.jl:1-24) on the FP32 pressure.
__global__ void k_sensor32(const DevParams P, const float* Q32, float* phi) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    cell_ijk(P, c, i, j, k);
    if (i < 1 || i > P.nxt - 2 || j < 1 || j > P.nyt - 2 || k < 1 || k > P.nzt - 2) return;
    const float* p = Q32 + 4 * P.plane;
    const long long sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const float pc = p[c];
    auto term = [](float a, float b, float d) { return fabsf(-a + 2.f * b - d) / (a + 2.f * b + d); };
    phi[c] = term(p[c - 1], pc, p[c + 1]) + term(p[c - sy], pc, p[c + sy]) + term(p[c - sz], pc, p[c + sz]);
}
cudaError_t launch_sensor32(const DevParams& P, const float* Q32, float* phi, cudaStream_t st) {
    k_sensor32<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q32, phi);
    return cudaGetLastError();
}

// FP32 copies of the metrics, |A_d|, A_d/|A_d| and J for the mixed form; |A_d| and A_d/|A_d|
// are formed in FP64 (the metric computation stays FP64) and rounded once.
__global__ void k_metric_prep32(const DevParams P, MetricPtrs m, MetricPtrs32 o) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double a = m.m[3 * d][c], b = m.m[3 * d + 1][c], e = m.m[3 * d + 2][c];
        const double s = sqrt(a * a + b * b + e * e);
        const double si = 1.0 / s;
        o.S[d][c] = (float)s;
        o.A[3 * d][c] = (float)a;
        o.A[3 * d + 1][c] = (float)b;
        o.A[3 * d + 2][c] = (float)e;
        o.H[3 * d][c] = (float)(a * si);
        o.H[3 * d + 1][c] = (float)(b * si);
        o.H[3 * d + 2][c] = (float)(e * si);
    }
    o.J[c] = (float)m.J[c];
}
cudaError_t launch_metric_prep32(const DevParams& P, const MetricPtrs& m, const MetricPtrs32& o, cudaStream_t st) {
    k_metric_prep32<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, m, o);
    return cudaGetLastError();
}

// utils.jl:2-30, interior only.
__global__ void k_c2prim(const DevParams P, const double* U, double* Q) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    cell_ijk(P, c, i, j, k);
    if (!is_interior(P, i, j, k)) return;
    double u[5], q[6];
#pragma unroll
    for (int n = 0; n < 5; n++) u[n] = U[c + n * P.plane];
    c2prim_cell(P, u, q);
#pragma unroll
    for (int n = 0; n < 6; n++) Q[c + n * P.plane] = q[n];
}
cudaError_t launch_c2prim_interior(const DevParams& P, const double* U, double* Q, cudaStream_t st) {
    k_c2prim<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, U, Q);
    return cudaGetLastError();
}

// utils.jl:33-54, every cell.
__global__ void k_prim2c(const DevParams P, const double* Q, double* U) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    double q[6], u[5];
#pragma unroll
    for (int n = 0; n < 6; n++) q[n] = Q[c + n * P.plane];
    prim2c_cell(P, q, u);
#pragma unroll
    for (int n = 0; n < 5; n++) U[c + n * P.plane] = u[n];
}
cudaError_t launch_prim2c(const DevParams& P, const double* Q, double* U, cudaStream_t st) {
    k_prim2c<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q, U);
    return cudaGetLastError();
}

// utils.jl:57-70, interior only.
__global__ void k_lincomb(const DevParams P, double* U, const double* Un, double a, double b) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    cell_ijk(P, c, i, j, k);
    if (!is_interior(P, i, j, k)) return;
#pragma unroll
    for (int n = 0; n < 5; n++) {
        const long long o = c + n * P.plane;
        U[o] = U[o] * a + Un[o] * b;
    }
}
cudaError_t launch_lincomb(const DevParams& P, double* U, const double* Un, double a, double b, cudaStream_t st) {
    k_lincomb<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, U, Un, a, b);
    return cudaGetLastError();
}

__global__ void k_sound(const DevParams P, const double* Q, double* csnd) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    double q[6];
#pragma unroll
    for (int n = 0; n < 6; n++) q[n] = Q[c + n * P.plane];
    csnd[c] = sound_speed(P, q);
}
cudaError_t launch_sound(const DevParams& P, const double* Q, double* csnd, cudaStream_t st) {
    k_sound<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q, csnd);
    return cudaGetLastError();
}

// schemes.jl:1-24 shockSensor at cells 2..Nt-1 (1-based), i.e. 1..Nt-2 here. The
// operation order matches the CPU restatement exactly so the branch map agrees bitwise.
__device__ __forceinline__ double sensor_term(double a, double b, double c) {
    double num = __dadd_rn(__dadd_rn(-a, __dmul_rn(2.0, b)), -c);
    double den = __dadd_rn(__dadd_rn(a, __dmul_rn(2.0, b)), c);
    return fabs(num) / den;
}
// EXACT: every cell's phi bit for bit as the oracle's (f3d_debug_sensor). Otherwise the
// sensor feeds only the branch of each face, i.e. comparisons of the largest phi of six cells
// with the thresholds phi1 < phi2 < phi3: phi is first formed in FP32 from the FP32-rounded
// pressures, and kept (widened exactly) when it lies more than a margin of 1e-5 max(1, t)
// from every threshold t and all seven pressures are positive; otherwise the FP64 value is
// computed as above. With positive pressures each of the three terms lies in [0, 1] and its
// FP32 evaluation is within 1e-6 of the exact value (pressure rounding 2^-24 relative, five
// FP32 roundings), so a kept value is on the same side of every threshold as the FP64 value:
// the branch map is the FP64 sensor's, with three FP64 divisions saved at almost every cell.
template <bool EXACT> __global__ void k_sensor(const DevParams P, const double* Q, double* phi) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    int i, j, k;
    cell_ijk(P, c, i, j, k);
    if (i < 1 || i > P.nxt - 2 || j < 1 || j > P.nyt - 2 || k < 1 || k > P.nzt - 2) return;
    const double* p = Q + 4 * P.plane;
    const long long sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const double pc = p[c], pxm = p[c - 1], pxp = p[c + 1], pym = p[c - sy], pyp = p[c + sy], pzm = p[c - sz],
                 pzp = p[c + sz];
    if (!EXACT) {
        const float b = f64_to_f32_rn(pc), xm = f64_to_f32_rn(pxm), xp = f64_to_f32_rn(pxp), ym = f64_to_f32_rn(pym),
                    yp = f64_to_f32_rn(pyp), zm = f64_to_f32_rn(pzm), zp = f64_to_f32_rn(pzp);
        const bool positive = b > 0.f && xm > 0.f && xp > 0.f && ym > 0.f && yp > 0.f && zm > 0.f && zp > 0.f;
        auto term = [](float a, float bb, float d) { return fabsf(-a + 2.f * bb - d) / (a + 2.f * bb + d); };
        const float f = term(xm, b, xp) + term(ym, b, yp) + term(zm, b, zp);
        const Cst<float>& K = P.cf;
        auto clear = [&](float t) { return fabsf(f - t) > 1e-5f * fmaxf(1.f, t); };
        if (positive && clear(K.phi1) && clear(K.phi2) && clear(K.phi3)) {
            phi[c] = f32_to_f64(f);
            return;
        }
    }
    double fx = sensor_term(pxm, pc, pxp);
    double fy = sensor_term(pym, pc, pyp);
    double fz = sensor_term(pzm, pc, pzp);
    phi[c] = __dadd_rn(__dadd_rn(fx, fy), fz);
}
cudaError_t launch_sensor(const DevParams& P, const double* Q, double* phi, cudaStream_t st, bool exact) {
    if (exact) k_sensor<true><<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q, phi);
    else k_sensor<false><<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q, phi);
    return cudaGetLastError();
}

// |grad xi_d| (solver.jl:286-288) and A_d * (1/|A_d|) (split.jl:28-32) for d = 0,1,2.
__global__ void k_metric_prep(const DevParams P, const double* m0, const double* m1, const double* m2,
                              const double* m3, const double* m4, const double* m5, const double* m6,
                              const double* m7, const double* m8, double* S0, double* S1, double* S2, double* H0,
                              double* H1, double* H2, double* H3, double* H4, double* H5, double* H6, double* H7,
                              double* H8) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    const double* m[9] = {m0, m1, m2, m3, m4, m5, m6, m7, m8};
    double* S[3] = {S0, S1, S2};
    double* H[9] = {H0, H1, H2, H3, H4, H5, H6, H7, H8};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double a = m[3 * d][c], b = m[3 * d + 1][c], e = m[3 * d + 2][c];
        const double s = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(e, e)));
        const double si = 1.0 / s;
        S[d][c] = s;
        H[3 * d][c] = a * si;
        H[3 * d + 1][c] = b * si;
        H[3 * d + 2][c] = e * si;
    }
}
cudaError_t launch_metric_prep(const DevParams& P, const double* const m[9], double* S[3], double* H[9],
                               cudaStream_t st) {
    k_metric_prep<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7],
                                                              m[8], S[0], S[1], S[2], H[0], H[1], H[2], H[3],
                                                              H[4], H[5], H[6], H[7], H[8]);
    return cudaGetLastError();
}

// fluxSplit_* at every cell into full (Nt^3 x 5) arrays (stage-by-stage parity).
__global__ void k_split_debug(const DevParams P, const double* Q, const double* csnd, const double* A0,
                              const double* A1, const double* A2, const double* H0, const double* H1,
                              const double* H2, const double* S, double* Fp, double* Fm) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.plane) return;
    double q[6], fp[5], fm[5];
#pragma unroll
    for (int n = 0; n < 6; n++) q[n] = Q[c + n * P.plane];
    split_cell<double>(P.split, P.cd, q, csnd[c], A0[c], A1[c], A2[c], H0[c], H1[c], H2[c], S[c], fp, fm);
#pragma unroll
    for (int n = 0; n < 5; n++) {
        Fp[c + n * P.plane] = fp[n];
        Fm[c + n * P.plane] = fm[n];
    }
}
cudaError_t launch_split_debug(const DevParams& P, const double* Q, const double* csnd, const double* const A[3],
                               const double* const H[3], const double* S, double* Fp, double* Fm, cudaStream_t st) {
    k_split_debug<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q, csnd, A[0], A[1], A[2], H[0], H[1], H[2], S,
                                                              Fp, Fm);
    return cudaGetLastError();
}

// div.jl:1-50 on caller arrays (the reference's own kernel boundary).
__global__ void k_div_ref(const DevParams P, double* U, const double* Fx, const double* Fy, const double* Fz,
                          const double* Fvx, const double* Fvy, const double* Fvz, const double* J, double dt) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nint = (long long)P.nx * P.ny * P.nz;
    if (t >= nint) return;
    int i, j, k;
    split3(t, P.dnx, P.dny, i, j, k);
    const long long c = lin3(P, i + NG, j + NG, k + NG);
    const double Jact = J[c] * dt;
    const long long fx = P.nx + 1, fy = P.ny + 1, fz = P.nz + 1;
    const long long nfx = fx * P.ny * P.nz, nfy = (long long)P.nx * fy * P.nz, nfz = (long long)P.nx * P.ny * fz;
    const long long ox = i + fx * (j + (long long)P.ny * k);
    const long long oy = i + (long long)P.nx * (j + fy * k);
    const long long oz = i + (long long)P.nx * (j + (long long)P.ny * k);
    const long long sz = (long long)P.nx * P.ny;
    double dv[4] = {0, 0, 0, 0};
    if (Fvx) {
        const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
        const long long vpl = (long long)vxt * vyt * vzt;
        const long long vc = (i + 2) + (long long)vxt * ((j + 2) + (long long)vyt * (k + 2));
        const long long sy = vxt, szz = (long long)vxt * vyt;
        const double c1 = 1.0 / 12.0, c2 = -2.0 / 3.0;
        for (int n = 0; n < 4; n++) {
            const double *X = Fvx + n * vpl + vc, *Y = Fvy + n * vpl + vc, *Z = Fvz + n * vpl + vc;
            double a = c1 * (X[-2] - X[2]) + c2 * (X[-1] - X[1]);
            double b = c1 * (Y[-2 * sy] - Y[2 * sy]) + c2 * (Y[-sy] - Y[sy]);
            double e = c1 * (Z[-2 * szz] - Z[2 * szz]) + c2 * (Z[-szz] - Z[szz]);
            dv[n] = a + b + e;
        }
    }
    for (int n = 0; n < 5; n++) {
        double inv = Fx[ox + n * nfx] - Fx[ox + 1 + n * nfx] + Fy[oy + n * nfy] - Fy[oy + P.nx + n * nfy] +
                     Fz[oz + n * nfz] - Fz[oz + sz + n * nfz];
        double u = U[c + n * P.plane] + inv * Jact;
        if (Fvx && n >= 1) u += dv[n - 1] * Jact;
        U[c + n * P.plane] = u;
    }
}
cudaError_t launch_div_ref(const DevParams& P, double* U, const double* Fx, const double* Fy, const double* Fz,
                           const double* Fvx, const double* Fvy, const double* Fvz, const double* J, double dt,
                           cudaStream_t st) {
    k_div_ref<<<pw_blocks((long long)P.nx * P.ny * P.nz), PW_THREADS, 0, st>>>(P, U, Fx, Fy, Fz, Fvx, Fvy, Fvz, J,
                                                                               dt);
    return cudaGetLastError();
}

// NaN/Inf scan of the interior of U (solver.jl:481-486).
__global__ void k_check_finite(const DevParams P, const double* U, int* flag) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    if (c < P.plane) {
        int i, j, k;
        cell_ijk(P, c, i, j, k);
        if (is_interior(P, i, j, k))
            for (int n = 0; n < 5; n++) bad |= !isfinite(U[c + n * P.plane]);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}
cudaError_t launch_check_finite(const DevParams& P, const double* U, int* flag, cudaStream_t st) {
    k_check_finite<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, U, flag);
    return cudaGetLastError();
}

// Global CFL time step: cfl * min over interior cells and directions of
// 1 / (J (|A_d . u| + c |A_d|)). Positive doubles order like their bit patterns, so the
// minimum is an atomicMin on the 64-bit pattern.
__global__ void k_cfl(const DevParams P, const double* Q, const double* m0, const double* m1, const double* m2,
                      const double* m3, const double* m4, const double* m5, const double* m6, const double* m7,
                      const double* m8, const double* J, double cfl, unsigned long long* out) {
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    double dt = __longlong_as_double(0x7ff0000000000000LL);  // +inf
    if (c < P.plane) {
        int i, j, k;
        cell_ijk(P, c, i, j, k);
        if (is_interior(P, i, j, k)) {
            const double rho = Q[c], u = Q[c + P.plane], v = Q[c + 2 * P.plane], w = Q[c + 3 * P.plane];
            const double T = Q[c + 5 * P.plane];
            const double a = sqrt(P.grg * T);
            const double* m[9] = {m0, m1, m2, m3, m4, m5, m6, m7, m8};
            double lam = 0.0;
            for (int d = 0; d < 3; d++) {
                const double A1 = m[3 * d][c], A2 = m[3 * d + 1][c], A3 = m[3 * d + 2][c];
                const double s = sqrt(A1 * A1 + A2 * A2 + A3 * A3);
                lam = fmax(lam, fabs(A1 * u + A2 * v + A3 * w) + a * s);
            }
            (void)rho;
            dt = cfl / (J[c] * lam);
        }
    }
    for (int o = 16; o > 0; o >>= 1) dt = fmin(dt, __shfl_xor_sync(0xffffffffu, dt, o));
    if ((threadIdx.x & 31) == 0 && dt > 0.0) atomicMin(out, (unsigned long long)__double_as_longlong(dt));
}
cudaError_t launch_cfl(const DevParams& P, const double* Q, const double* const m[9], const double* J, double cfl,
                       unsigned long long* out, cudaStream_t st) {
    k_cfl<<<pw_blocks(P.plane), PW_THREADS, 0, st>>>(P, Q, m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8], J,
                                                      cfl, out);
    return cudaGetLastError();
}

// ---- pipe throughput probe ------------------------------------------------------------
template <class T>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int c = 0; c < 8; c++) x[c] = (T)(threadIdx.x + c);
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int c = 0; c < 8; c++) x[c] = x[c] * a + b;
    }
    T s = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) s += x[c];
    out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class T> static double time_fma(int blocks, int threads, int iters, T* buf) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_chain<T><<<blocks, threads>>>(buf, iters, (T)0.999999, (T)1e-7);
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(e0);
        k_fma_chain<T><<<blocks, threads>>>(buf, iters, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = ms < best ? ms : best;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * (double)blocks * threads * 8.0 * iters;
    return flops / (best * 1e-3) / 1e12;
}

cudaError_t measure_pipes(double* fp64, double* fp32) {
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = nsm * 8, threads = 256;
    void* buf = nullptr;
    e = cudaMalloc(&buf, (size_t)blocks * threads * sizeof(double));
    if (e != cudaSuccess) return e;
    *fp64 = time_fma<double>(blocks, threads, 2000, (double*)buf);
    *fp32 = time_fma<float>(blocks, threads, 40000, (float*)buf);
    e = cudaGetLastError();
    cudaFree(buf);
    return e;
}

}  // namespace f3d
