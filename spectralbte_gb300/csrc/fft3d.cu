// fft3d.cu -- batched phase-shifted 3D DFT (the reference's fft3D,
// collisions.c:232-283).
//
// The reference brackets an unnormalised FFTW transform with two phase
// loops (collisions.c:257-268 and 273-281).  Both phase factors and the
// trapezoid weights separate by axis.  So the whole operator is
// prefactor * (D (x) D (x) D), where D is one dense N x N complex matrix
// built once on the host in FP64 (see kernels.h).  Each launch applies D
// along the contiguous axis and the middle axis of one plane, entirely in
// shared memory.  A second launch applies it along the slow axis.  At the
// sizes of this code (N <= 64) the dense O(N^4) form costs about 0.3% of one
// convolution at N = 32.  It needs no radix restriction, so N = 24 and odd N
// take the same path.
#include "common.cuh"
#include "kernels.h"

namespace sbte {
namespace {

template <typename T> struct Cx;
template <> struct Cx<double> { using t = double2; };
template <> struct Cx<float> { using t = float2; };

__device__ __forceinline__ long long lay(int b, long long pos, long long n3,
                                         int bg)
{
    return (long long)(b / bg) * n3 * bg + pos * bg + (b % bg);
}

template <typename T>
__device__ __forceinline__ typename Cx<T>::t load_in(const void *p,
                                                     DftIn kind, long long i)
{
    typename Cx<T>::t r;
    if (kind == DftIn::kRealF64) {
        r.x = (T)(static_cast<const double *>(p)[i]);
        r.y = (T)0;
    } else if (kind == DftIn::kComplexF64) {
        double2 d = static_cast<const double2 *>(p)[i];
        r.x = (T)d.x;
        r.y = (T)d.y;
    } else {
        float2 d = static_cast<const float2 *>(p)[i];
        r.x = (T)d.x;
        r.y = (T)d.y;
    }
    return r;
}

template <typename T>
__device__ __forceinline__ void store_out(void *p, DftOut kind, long long i,
                                          typename Cx<T>::t v)
{
    switch (kind) {
    case DftOut::kComplexF64:
        static_cast<double2 *>(p)[i] = make_double2((double)v.x, (double)v.y);
        break;
    case DftOut::kComplexF32:
        static_cast<float2 *>(p)[i] = make_float2((float)v.x, (float)v.y);
        break;
    case DftOut::kRealF64:
        static_cast<double *>(p)[i] = (double)v.x;
        break;
    case DftOut::kRealF32:
        static_cast<float *>(p)[i] = (float)v.x;
        break;
    case DftOut::kF4:
        static_cast<float4 *>(p)[i] = make_float4((float)v.x, (float)v.y, (float)v.y, (float)v.x);
        break;
    case DftOut::kG4:
        static_cast<float4 *>(p)[i] =
            make_float4((float)v.x, (float)v.x, -(float)v.y, (float)v.y);
        break;
    }
}

// Complex multiply-accumulate acc += a * b.
template <typename C2>
__device__ __forceinline__ void cmac(C2 &acc, C2 a, C2 b)
{
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}

// Plane pass: for instance b = blockIdx.y and slow index i = blockIdx.x,
// transform the (j, k) plane along k, then along j.
template <typename T>
__global__ void __launch_bounds__(256)
dft_plane(const void *__restrict__ in, DftIn in_kind, int in_bg,
          typename Cx<T>::t *__restrict__ tmp, const typename Cx<T>::t *__restrict__ Dt,
          int N)
{
    using C2 = typename Cx<T>::t;
    extern __shared__ unsigned char smem_raw[];
    C2 *sD = reinterpret_cast<C2 *>(smem_raw);
    C2 *sX = sD + N * N;
    C2 *sZ = sX + N * N;
    const int i = blockIdx.x, b = blockIdx.y, nn = N * N;
    const long long n3 = (long long)nn * N;
    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
        sD[t] = Dt[t];
        sX[t] = load_in<T>(in, in_kind, lay(b, (long long)i * nn + t, n3, in_bg));
    }
    __syncthreads();
    // along k: Z[j][k] = sum_n D[k][n] X[j][n]
    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
        int j = t / N, k = t - j * N;
        C2 acc;
        acc.x = 0;
        acc.y = 0;
        for (int n = 0; n < N; n++) cmac(acc, sD[n * N + k], sX[j * N + n]);
        sZ[t] = acc;
    }
    __syncthreads();
    // along j: Y[j'][k] = sum_j D[j'][j] Z[j][k]
    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
        int jp = t / N, k = t - jp * N;
        C2 acc;
        acc.x = 0;
        acc.y = 0;
        for (int j = 0; j < N; j++) cmac(acc, sD[j * N + jp], sZ[j * N + k]);
        tmp[(long long)b * n3 + (long long)i * nn + t] = acc;
    }
}

// Pencil pass: for instance b = blockIdx.y and middle index j = blockIdx.x,
// transform along the slow axis i and apply the prefactor.
template <typename T>
__global__ void __launch_bounds__(256)
dft_pencil(const typename Cx<T>::t *__restrict__ tmp, void *__restrict__ out,
           DftOut out_kind, int out_bg, const typename Cx<T>::t *__restrict__ Dt,
           T prefactor, int N)
{
    using C2 = typename Cx<T>::t;
    extern __shared__ unsigned char smem_raw[];
    C2 *sD = reinterpret_cast<C2 *>(smem_raw);
    C2 *sY = sD + N * N;  // sY[i][k] = tmp[i][j][k]
    const int j = blockIdx.x, b = blockIdx.y, nn = N * N;
    const long long n3 = (long long)nn * N;
    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
        sD[t] = Dt[t];
        int i = t / N, k = t - i * N;
        sY[t] = tmp[(long long)b * n3 + (long long)i * nn + (long long)j * N + k];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < nn; t += blockDim.x) {
        int ip = t / N, k = t - ip * N;
        C2 acc;
        acc.x = 0;
        acc.y = 0;
        for (int i = 0; i < N; i++) cmac(acc, sD[i * N + ip], sY[i * N + k]);
        acc.x *= prefactor;
        acc.y *= prefactor;
        store_out<T>(out, out_kind,
                     lay(b, (long long)ip * nn + (long long)j * N + k, n3, out_bg), acc);
    }
}

template <typename T>
cudaError_t dft3_impl(const void *in, DftIn in_kind, int in_bg,
                      typename Cx<T>::t *tmp, void *out, DftOut out_kind,
                      int out_bg, const typename Cx<T>::t *Dt, T prefactor,
                      int N, int B, cudaStream_t st)
{
    using C2 = typename Cx<T>::t;
    if (N < 2 || N > 64 || B < 1 || B > 65535) return cudaErrorInvalidValue;
    size_t sm_plane = 3 * sizeof(C2) * N * N;
    size_t sm_pencil = 2 * sizeof(C2) * N * N;
    if (sm_plane > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(
            dft_plane<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm_plane);
        if (e != cudaSuccess) return e;
        e = cudaFuncSetAttribute(dft_pencil<T>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sm_pencil);
        if (e != cudaSuccess) return e;
    }
    dim3 grid(N, B);
    dft_plane<T><<<grid, 256, sm_plane, st>>>(in, in_kind, in_bg, tmp, Dt, N);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dft_pencil<T><<<grid, 256, sm_pencil, st>>>(tmp, out, out_kind, out_bg, Dt,
                                                prefactor, N);
    return cudaGetLastError();
}

}  // namespace

cudaError_t dft3_f64(const void *in, DftIn in_kind, int in_bg, double2 *tmp,
                     void *out, DftOut out_kind, int out_bg,
                     const double2 *Dt, double prefactor, int N, int B,
                     cudaStream_t st)
{
    return dft3_impl<double>(in, in_kind, in_bg, tmp, out, out_kind, out_bg,
                             Dt, prefactor, N, B, st);
}

cudaError_t dft3_f32(const void *in, DftIn in_kind, int in_bg, float2 *tmp,
                     void *out, DftOut out_kind, int out_bg, const float2 *Dt,
                     float prefactor, int N, int B, cudaStream_t st)
{
    return dft3_impl<float>(in, in_kind, in_bg, tmp, out, out_kind, out_bg,
                            Dt, prefactor, N, B, st);
}

}  // namespace sbte
