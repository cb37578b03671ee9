// fma_probe.cu -- roofline calibration for the benchmark: the FP32 FMA rate
// this GPU sustains.  Built into its own library, libspectral_calib.so, which
// only the benchmark loads; the collision library does not contain it.
//
// The FP32 convolution is bound by FP32 FMA issue.  The nominal peak (SMs x
// 128 lanes x 2 flop x maximum clock) assumes the maximum clock, and the clock
// under a dense FMA load sits below it.  This probe runs independent FMA
// chains held in registers, the most favourable FP32 instruction stream, and
// reports the sustained rate.  The benchmark divides by it.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) fma_probe_kernel(float *out, int iters, float a, float b)
{
    float r[16];
#pragma unroll
    for (int i = 0; i < 16; i++) r[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int i = 0; i < 16; i++) r[i] = fmaf(r[i], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < 16; i++) s += r[i];
    if (s == 1234.5f) out[threadIdx.x] = s;  // keeps the chains live
}

}  // namespace

// FP32 FMA rate (TFLOP/s, one FMA = 2 flop) of the current device on
// `stream` (NULL: default stream).  Returns 0, or the cudaError_t of the
// failing call.
extern "C" int spectral_calib_fp32_fma_rate(double *tflops, void *stream)
{
    if (!tflops) return (int)cudaErrorInvalidValue;
    int dev = 0, nsm = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return (int)e;
    cudaStream_t st = (cudaStream_t)stream;
    float *sink = nullptr;
    if ((e = cudaMalloc(&sink, 256 * sizeof(float))) != cudaSuccess) return (int)e;
    const int blocks = nsm * 8, threads = 256, iters = 1 << 15;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    if (e == cudaSuccess) {
        fma_probe_kernel<<<blocks, threads, 0, st>>>(sink, 1024, 0.999f, 0.001f);  // warm-up
        cudaEventRecord(e0, st);
        fma_probe_kernel<<<blocks, threads, 0, st>>>(sink, iters, 0.999f, 0.001f);
        cudaEventRecord(e1, st);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return (int)e;
    const double fmas = (double)blocks * threads * iters * 16;
    *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
    return 0;
}
