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
    int vi, vj, vk;
    split3(t, P.dvxt, P.dvyt, vi, vj, vk);
    const long long c = lin3(P, vi + 2, vj + 2, vk + 2);
    const long long pl = P.plane, sy = P.nxt, sz = (long long)P.nxt * P.nyt;
    const Cst<R>& K = cst<R>(P);
    const R xx = m0[c], xy = m1[c], xz = m2[c];
    const R ex = m3[c], ey = m4[c], ez = m5[c];
    const R zx = m6[c], zy = m7[c], zz = m8[c];
    const R Jac = J[c];
    const R T = Q[c + 5 * pl];
    R mu = K.c_s * T * sqrt(T) / (T + K.t_s);
    R lam = mu * K.cp_pr;
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
    if (P.les) {  // viscous.jl:66-106: eddy viscosity and conductivity, Pr_t = 0.9
        const R rho = Q[c];
        const R s12 = R(0.5) * (dudy + dvdx), s13 = R(0.5) * (dudz + dwdx), s23 = R(0.5) * (dvdz + dwdy);
        const R sii = dudx * dudx + dvdy * dvdy + dwdz * dwdz;
        const R sij = s12 * s12 + s13 * s13 + s23 * s23;
        const R inv_d = R(1) / cbrt(Jac);  // 1 / Delta with Delta = J^(1/3) (cell size, J^-1 = volume)
        R mut;
        if (P.les == F3D_LES_SMAGORINSKY) {
            const R Smag = sqrt(R(2) * (sii + R(2) * sij));  // sqrt(2) |S_ij|
            const R cd = R(0.1) * inv_d;
            mut = rho * cd * cd * Smag;
        } else {  // WALE
            const R S = sqrt(sii + R(2) * sij);
            R d11 = dudx * dudx + dudy * dvdx + dudz * dwdx;
            R d22 = dvdx * dudy + dvdy * dvdy + dvdz * dwdy;
            R d33 = dwdx * dudz + dwdy * dvdz + dwdz * dwdz;
            const R tr = R(1) / R(3) * (d11 + d22 + d33);
            d11 -= tr;
            d22 -= tr;
            d33 -= tr;
            const R d12 = R(0.5) * (dudx * dvdx + dvdx * dvdy + dwdx * dvdz + dudy * dudx + dvdy * dudy + dwdy * dudz);
            const R d13 = R(0.5) * (dudx * dwdx + dvdx * dwdy + dwdx * dwdz + dudz * dudx + dvdz * dudy + dwdz * dudz);
            const R d23 = R(0.5) * (dudy * dwdx + dvdy * dwdy + dwdy * dwdz + dudz * dvdx + dvdz * dvdy + dwdz * dvdz);
            const R Sd = sqrt(d11 * d11 + d22 * d22 + d33 * d33 + R(2) * (d12 * d12 + d13 * d13 + d23 * d23));
            const R S2 = S * S;
            const R D = Sd * Sd * Sd / (S2 * S2 * S + Sd * Sd * sqrt(Sd));
            const R cd = R(0.325) * inv_d;
            mut = rho * cd * cd * D;
        }
        // min(mu_t, 2 mu) returning NaN when either is NaN, as Julia's min does (D = 0/0 where
        // the velocity gradient vanishes)
        const R lim = R(2) * mu;
        mut = (mut != mut) ? mut : (lim < mut ? lim : mut);
        mu += mut;
        lam += K.cp * mut / R(0.9);
    }
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
