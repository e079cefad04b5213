// k_viscous.cu — viscous and heat fluxes (viscous.jl:1-64, 107-133; the LES branches at
// viscous.jl:66-106 are off in the reference configuration and not built).
//
// One thread per cell of the box 2..Nt-3 (0-based full index), which is cells 3..Nt-2 of
// the reference. Fourth-order central differences of u, v, w, T in xi, eta, zeta, the
// chain rule with the J^-1-scaled metrics and J, Sutherland viscosity, Stokes stress and
// Fourier heat flux, projected on the three metric rows. Output arrays have the
// reference's Fv_x/Fv_y/Fv_z shape ((Nt-4)^3 x 4) with Fv index = cell index - 2.
#include "f3d_kernels.cuh"

namespace f3d {

template <class R>
__global__ void __launch_bounds__(128) k_viscous(const DevParams P, const R* __restrict__ Q, const R* m0,
                                                 const R* m1, const R* m2, const R* m3, const R* m4, const R* m5,
                                                 const R* m6, const R* m7, const R* m8, const R* __restrict__ J,
                                                 R* Fvx, R* Fvy, R* Fvz) {
    const int vxt = P.nxt - 4, vyt = P.nyt - 4, vzt = P.nzt - 4;
    const long long vpl = (long long)vxt * vyt * vzt;
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= vpl) return;
    const int vi = (int)(t % vxt), vj = (int)((t / vxt) % vyt), vk = (int)(t / ((long long)vxt * vyt));
    const long long c = lin3(P, vi + 2, vj + 2, vk + 2);
    const long long pl = P.plane, sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const Cst<R>& K = cst<R>(P);
    const R xx = m0[c], xy = m1[c], xz = m2[c];
    const R ex = m3[c], ey = m4[c], ez = m5[c];
    const R zx = m6[c], zy = m7[c], zz = m8[c];
    const R Jac = J[c];
    const R T = Q[c + 5 * pl];
    const R mu = K.c_s * T * sqrt(T) / (T + K.t_s);
    const R lam = mu * K.cp_pr;
    const R c1 = R(1) / R(12), c2 = R(-2) / R(3), c23 = R(2) / R(3);
    auto d4 = [&](int n, long long s) {
        const R* f = Q + n * pl + c;
        return c1 * (f[-2 * s] - f[2 * s]) + c2 * (f[-s] - f[s]);
    };
    // viscous.jl:29-42: the CD4 coefficients give +d/dxi
    const R uxi = d4(1, 1), vxi = d4(2, 1), wxi = d4(3, 1), Txi = d4(5, 1);
    const R uet = d4(1, sy), vet = d4(2, sy), wet = d4(3, sy), Tet = d4(5, sy);
    const R uze = d4(1, sz), vze = d4(2, sz), wze = d4(3, sz), Tze = d4(5, sz);
    const R u = Q[c + pl], v = Q[c + 2 * pl], w = Q[c + 3 * pl];
    const R dudx = (uxi * xx + uet * ex + uze * zx) * Jac;
    const R dudy = (uxi * xy + uet * ey + uze * zy) * Jac;
    const R dudz = (uxi * xz + uet * ez + uze * zz) * Jac;
    const R dvdx = (vxi * xx + vet * ex + vze * zx) * Jac;
    const R dvdy = (vxi * xy + vet * ey + vze * zy) * Jac;
    const R dvdz = (vxi * xz + vet * ez + vze * zz) * Jac;
    const R dwdx = (wxi * xx + wet * ex + wze * zx) * Jac;
    const R dwdy = (wxi * xy + wet * ey + wze * zy) * Jac;
    const R dwdz = (wxi * xz + wet * ez + wze * zz) * Jac;
    const R dTdx = (Txi * xx + Tet * ex + Tze * zx) * Jac;
    const R dTdy = (Txi * xy + Tet * ey + Tze * zy) * Jac;
    const R dTdz = (Txi * xz + Tet * ez + Tze * zz) * Jac;
    const R dv = dudx + dvdy + dwdz;
    const R t11 = mu * (R(2) * dudx - c23 * dv);
    const R t12 = mu * (dudy + dvdx);
    const R t13 = mu * (dudz + dwdx);
    const R t22 = mu * (R(2) * dvdy - c23 * dv);
    const R t23 = mu * (dwdy + dvdz);
    const R t33 = mu * (R(2) * dwdz - c23 * dv);
    const R E1 = u * t11 + v * t12 + w * t13 + lam * dTdx;
    const R E2 = u * t12 + v * t22 + w * t23 + lam * dTdy;
    const R E3 = u * t13 + v * t23 + w * t33 + lam * dTdz;
    Fvx[t] = xx * t11 + xy * t12 + xz * t13;
    Fvx[t + vpl] = xx * t12 + xy * t22 + xz * t23;
    Fvx[t + 2 * vpl] = xx * t13 + xy * t23 + xz * t33;
    Fvx[t + 3 * vpl] = xx * E1 + xy * E2 + xz * E3;
    Fvy[t] = ex * t11 + ey * t12 + ez * t13;
    Fvy[t + vpl] = ex * t12 + ey * t22 + ez * t23;
    Fvy[t + 2 * vpl] = ex * t13 + ey * t23 + ez * t33;
    Fvy[t + 3 * vpl] = ex * E1 + ey * E2 + ez * E3;
    Fvz[t] = zx * t11 + zy * t12 + zz * t13;
    Fvz[t + vpl] = zx * t12 + zy * t22 + zz * t23;
    Fvz[t + 2 * vpl] = zx * t13 + zy * t23 + zz * t33;
    Fvz[t + 3 * vpl] = zx * E1 + zy * E2 + zz * E3;
}

template <class R>
static cudaError_t launch_visc(const DevParams& P, const R* Q, const R* const m[9], const R* J, R* Fvx, R* Fvy,
                               R* Fvz, cudaStream_t st) {
    const long long n = (long long)(P.nxt - 4) * (P.nyt - 4) * (P.nzt - 4);
    k_viscous<R><<<(unsigned)((n + 127) / 128), 128, 0, st>>>(P, Q, m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7],
                                                              m[8], J, Fvx, Fvy, Fvz);
    return cudaGetLastError();
}
cudaError_t launch_viscous(const DevParams& P, const double* Q, const double* const m[9], const double* J,
                           double* Fvx, double* Fvy, double* Fvz, cudaStream_t st) {
    return launch_visc<double>(P, Q, m, J, Fvx, Fvy, Fvz, st);
}
cudaError_t launch_viscous32(const DevParams& P, const float* Q, const float* const m[9], const float* J,
                             float* Fvx, float* Fvy, float* Fvz, cudaStream_t st) {
    return launch_visc<float>(P, Q, m, J, Fvx, Fvy, Fvz, st);
}

}  // namespace f3d
