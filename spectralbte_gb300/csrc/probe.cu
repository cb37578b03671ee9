// probe.cu -- roofline calibration: the FP32 FMA rate this GPU sustains.
//
// The convolution is bound by FP32 FMA issue.  The nominal peak (SMs x 128
// lanes x 2 flop x maximum clock) assumes the maximum clock, and the clock
// under a dense FMA load sits below it.  This probe runs independent FMA
// chains held in registers, the most favourable FP32 instruction stream, and
// reports the sustained rate.  The benchmark divides by it.
#include "common.cuh"
#include "../../include/spectral_bte.h"

namespace sbte {
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
}  // namespace sbte

using namespace sbte;

extern "C" int spectral_fp32_fma_rate(double *tflops, void *stream)
{
    if (!tflops) return set_error(kErrArg, "null argument"), kErrArg;
    int dev = 0, nsm = 0;
    SBTE_CUDA(cudaGetDevice(&dev));
    SBTE_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    cudaStream_t st = (cudaStream_t)stream;
    float *sink = nullptr;
    SBTE_CUDA(cudaMalloc(&sink, 256 * sizeof(float)));
    const int blocks = nsm * 8, threads = 256, iters = 1 << 15;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_probe_kernel<<<blocks, threads, 0, st>>>(sink, 1024, 0.999f, 0.001f);  // warm-up
    cudaEventRecord(e0, st);
    fma_probe_kernel<<<blocks, threads, 0, st>>>(sink, iters, 0.999f, 0.001f);
    cudaEventRecord(e1, st);
    cudaError_t e = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    if (e != cudaSuccess) return set_error(kErrCuda, "fma probe: %s", cudaGetErrorString(e)), kErrCuda;
    const double fmas = (double)blocks * threads * iters * 16;
    *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
    return kOk;
}
