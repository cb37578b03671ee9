// noalloc.cu -- a batched 3D transform (the reference's fft3D,
// collisions.c:232-283) that allocates no device memory.
//
// Who needs it: a solver coupled into a host application that owns all
// device memory through its own pool, or a step inside a time-critical loop.
// In both, a cudaMalloc from this library would contend with the owner's
// allocator or stall the loop.  The caller passes its own input and output
// buffers.  The transform's only other storage lives in one fixed device
// array of this file: the axis matrix and the plane-pass intermediate.
// Every GPU that loads the library holds that array until the process
// exits.
#include "common.cuh"
#include "kernels.h"
#include "../../include/spectral_bte.h"

#include <cmath>
#include <mutex>

namespace sbte {
namespace {

// 32 MiB: room for the N x N axis matrix plus B*N^3 complex intermediates.
constexpr size_t kNoAllocElems = (size_t)1 << 21;  // double2 values
__device__ __align__(256) double2 g_noalloc_scratch[kNoAllocElems];

constexpr int kMaxDevices = 64;
double2 *g_noalloc_ptr[kMaxDevices] = {};
std::mutex g_noalloc_mu;

struct AxisSpec {
    int N;
    double sign, L_end, L_start, delta, fsign;
    double varr[64];
};

// Dt[n*N + k] = D[k][n] = wt[n] e^{i s L_end varr[k]} e^{i fs 2 pi (nk mod N)/N}
//                         e^{i s n L_start delta}
__global__ void axis_matrix_kernel(double2 *__restrict__ Dt, AxisSpec a)
{
    const int N = a.N;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < N * N;
         t += gridDim.x * blockDim.x) {
        const int n = t / N, k = t - n * N;
        const double ap = a.sign * a.L_end * a.varr[k];
        const double ad = a.fsign * 2.0 * M_PI * (double)((n * k) % N) / (double)N;
        const double aq = a.sign * (double)n * a.L_start * a.delta;
        double ci, cr, ti, tr, ui, ur;
        sincos(ap, &ci, &cr);
        sincos(ad, &ti, &tr);
        sincos(aq, &ui, &ur);
        const double r1 = cr * tr - ci * ti, i1 = cr * ti + ci * tr;
        const double r2 = r1 * ur - i1 * ui, i2 = r1 * ui + i1 * ur;
        const double w = (n == 0 || n == N - 1) ? 0.5 : 1.0;
        Dt[t] = make_double2(w * r2, w * i2);
    }
}

}  // namespace
}  // namespace sbte

using namespace sbte;

extern "C" int spectral_fft3d_noalloc(int N, double L_v, const double *v,
                                      const double *zeta, const double *in_dev,
                                      double *out_dev, int B, int invert,
                                      void *stream)
{
    if (N < 2 || N > 64 || B < 1 || !v || !zeta || !in_dev || !out_dev) {
        set_error(kErrArg, "spectral_fft3d_noalloc: bad arguments");
        return kErrArg;
    }
    const size_t need = (size_t)N * N + (size_t)B * N * N * N;
    if (need > kNoAllocElems) {
        set_error(kErrArg,
                  "spectral_fft3d_noalloc: B*N^3 + N^2 = %zu complex values exceeds the "
                  "32 MiB static scratch (%zu values)",
                  need, kNoAllocElems);
        return kErrArg;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        set_error(kErrCuda, "spectral_fft3d_noalloc: no current device (%s)",
                  cudaGetErrorString(e));
        return kErrCuda;
    }
    double2 *scratch = nullptr;
    {
        // Once per device, with that device current: the device address of
        // the static array (the host-side name is not a device address).
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
            if (e != cudaSuccess || !p) {
                set_error(kErrCuda, "spectral_fft3d_noalloc: cudaGetSymbolAddress: %s",
                          cudaGetErrorString(e));
                return kErrCuda;
            }
            g_noalloc_ptr[dev] = static_cast<double2 *>(p);
        }
        scratch = g_noalloc_ptr[dev];
    }
    // Module quantities as initialize_coll derives them (collisions.c:36-46)
    // and the direction choice of fft3D (collisions.c:238-253).
    AxisSpec a;
    a.N = N;
    const double dv = v[1] - v[0], deta = zeta[1] - zeta[0], L_eta = -zeta[0];
    const double *varr;
    if (!invert) {
        a.delta = dv; a.L_start = L_eta; a.L_end = L_v; varr = zeta; a.sign = 1.0; a.fsign = -1.0;
    } else {
        a.delta = deta; a.L_start = L_v; a.L_end = L_eta; varr = v; a.sign = -1.0; a.fsign = 1.0;
    }
    for (int k = 0; k < N; k++) a.varr[k] = varr[k];
    const double prefactor = pow(1.0 / sqrt(2.0 * M_PI), 3.0) * a.delta * a.delta * a.delta;

    cudaStream_t st = (cudaStream_t)stream;  // NULL: the default stream
    double2 *Dt = scratch;
    double2 *tmp = scratch + (size_t)N * N;
    axis_matrix_kernel<<<(N * N + 255) / 256, 256, 0, st>>>(Dt, a);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = dft3_f64(in_dev, DftIn::kComplexF64, 1, tmp, out_dev, DftOut::kComplexF64, 1, Dt,
                     prefactor, N, B, st);
    if (e != cudaSuccess) {
        set_error(kErrCuda, "spectral_fft3d_noalloc: %s", cudaGetErrorString(e));
        return kErrCuda;
    }
    return kOk;
}
