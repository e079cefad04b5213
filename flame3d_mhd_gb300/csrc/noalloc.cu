// noalloc.cu — f3d_rhs_noalloc: the right-hand side without any device allocation.
//
// f3d_rhs needs a context, and f3d_create obtains the context's scratch with cudaMalloc.
// Some callers cannot allocate device memory: hosts whose memory pool has reserved the
// device's memory and forbids foreign cudaMalloc/cudaFree (a framework allocator, or a job
// held to a fixed device-memory quota), and time-critical loops that cannot afford
// cudaFree's implicit synchronisation of the whole device. f3d_rhs_noalloc serves them: it takes the parameters,
// metrics and arrays directly, and keeps its scratch in one file-scope __device__ array of
// F3D_NOALLOC_SCRATCH_BYTES that the module holds on every GPU that loads the library,
// until the process exits.
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "f3d_kernels.cuh"

namespace f3d {

// The shared scratch. Host code must not use the name as an address: on the host it is a
// stand-in symbol, so its device address is looked up once per device with
// cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[F3D_NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Once per device, with that device current: the device address of the scratch array and
// the shared-memory attributes of the sweep kernels.
int setup_device(int dev, void** addr) {
    if (dev < 0 || dev >= kMaxDevices) return F3D_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) {
            std::fprintf(stderr, "f3d_rhs_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorString(e));
            return F3D_ERR_CUDA;
        }
        e = sweep_configure();
        if (e != cudaSuccess) {
            std::fprintf(stderr, "f3d_rhs_noalloc: kernel set-up failed: %s\n", cudaGetErrorString(e));
            return F3D_ERR_CUDA;
        }
        g_scratch_addr[dev] = p;
    }
    *addr = g_scratch_addr[dev];
    return F3D_OK;
}

bool aligned16(const void* p) { return p && ((uintptr_t)p & 15u) == 0; }

}  // namespace
}  // namespace f3d

using namespace f3d;

extern "C" int f3d_rhs_noalloc(const f3d_params* p, const double* const metrics[9], const double* jac,
                               const double* Q, double* dUdt, f3d_stream stream) {
    if (!p || !metrics) return F3D_ERR_ARG;
    std::string why;
    int rc = validate_params(*p, why);
    if (rc) {
        std::fprintf(stderr, "f3d_rhs_noalloc: %s\n", why.c_str());
        return rc;
    }
    if (p->scheme != F3D_SCHEME_FDM) {
        std::fprintf(stderr, "f3d_rhs_noalloc: the finite-volume schemes need a context (coordinates)\n");
        return F3D_ERR_UNSUPPORTED;
    }
    for (int f = 0; f < 6; f++)
        if (p->bc[f].kind == F3D_BC_INFLOW_PROFILE) {
            std::fprintf(stderr, "f3d_rhs_noalloc: inflow-profile faces need a context\n");
            return F3D_ERR_UNSUPPORTED;
        }
    if (p->precision != F3D_PREC_FP64) {
        std::fprintf(stderr, "f3d_rhs_noalloc: only the FP64 form is available without a context\n");
        return F3D_ERR_UNSUPPORTED;
    }
    for (int n = 0; n < 9; n++)
        if (!aligned16(metrics[n])) return F3D_ERR_ALIGN;
    if (!aligned16(jac) || !aligned16(Q) || !aligned16(dUdt)) return F3D_ERR_ALIGN;

    const DevParams P = make_dev_params(*p);
    // scratch: |A| (3), A/|A| (9), sound speed, sensor, and the viscous fluxes (3 x 4)
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t b1 = up((size_t)P.plane * sizeof(double));
    const size_t bv = up((size_t)(p->nx + 4) * (p->ny + 4) * (p->nz + 4) * 4 * sizeof(double));
    const size_t need = 14 * b1 + (p->viscous ? 3 * bv : 0);
    if (need > (size_t)F3D_NOALLOC_SCRATCH_BYTES) {
        std::fprintf(stderr,
                     "f3d_rhs_noalloc: grid %dx%dx%d needs %zu bytes of scratch, above the %d-byte limit "
                     "(F3D_NOALLOC_SCRATCH_BYTES); use f3d_create/f3d_rhs for this grid\n",
                     p->nx, p->ny, p->nz, need, F3D_NOALLOC_SCRATCH_BYTES);
        return F3D_ERR_TOO_LARGE;
    }
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return F3D_ERR_CUDA;
    void* base = nullptr;
    if ((rc = setup_device(dev, &base))) return rc;

    char* q = static_cast<char*>(base);
    double *S[3], *Ah[9], *csnd, *phi, *Fv[3] = {nullptr, nullptr, nullptr};
    for (int d = 0; d < 3; d++) { S[d] = (double*)q; q += b1; }
    for (int n = 0; n < 9; n++) { Ah[n] = (double*)q; q += b1; }
    csnd = (double*)q; q += b1;
    phi = (double*)q; q += b1;
    if (p->viscous)
        for (int d = 0; d < 3; d++) { Fv[d] = (double*)q; q += bv; }

    cudaStream_t st = (cudaStream_t)stream;
    const double* m[9];
    for (int n = 0; n < 9; n++) m[n] = metrics[n];
    cudaError_t e;
#define NA_CUDA(call)                                                                     \
    do {                                                                                  \
        if ((e = (call)) != cudaSuccess) {                                                \
            std::fprintf(stderr, "f3d_rhs_noalloc: %s: %s\n", #call, cudaGetErrorString(e)); \
            return F3D_ERR_CUDA;                                                          \
        }                                                                                 \
    } while (0)
    // the array keeps the previous call's contents: the sensor writes cells 1..Nt-2 only,
    // so its array starts from zero on every call
    NA_CUDA(cudaMemsetAsync(phi, 0, b1, st));
    NA_CUDA(launch_metric_prep(P, m, S, Ah, st));
    NA_CUDA(launch_sound(P, Q, csnd, st));
    const bool hybrid = P.fixed_branch < 0;
    if (hybrid) NA_CUDA(launch_sensor(P, Q, phi, st));
    if (p->viscous) NA_CUDA(launch_viscous(P, Q, m, jac, Fv[0], Fv[1], Fv[2], st));
    for (int d = 0; d < 3; d++) {
        SweepArgs a;
        std::memset(&a, 0, sizeof(a));
        a.P = P;
        a.Q = Q;
        a.csnd = csnd;
        for (int n = 0; n < 3; n++) {
            a.A[n] = m[3 * d + n];
            a.Ah[n] = Ah[3 * d + n];
        }
        a.S = S[d];
        a.phi = hybrid ? phi : nullptr;
        a.Fv = Fv[d];
        a.J = jac;
        a.acc = dUdt;  // dUdt accumulates the three directions
        a.out = dUdt;
        a.out_mode = d == 0 ? OUT_SET : (d == 1 ? OUT_ADD : OUT_RHS);
        NA_CUDA(launch_sweep(d, a, st));
    }
#undef NA_CUDA
    return F3D_OK;
}
