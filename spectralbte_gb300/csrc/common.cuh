// common.cuh -- shared host/device helpers for the GB300 collision library.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>

namespace sbte {

// Status codes returned by the spectral_* entry points and recorded for
// spectral_last_error().  They mirror the exit() paths of the reference:
// a short weight read (weights.c:83-86), a missing anisotropic weight file
// (weights.c:95-97) and a singular CC^T (conserve.c:130-135).  The library
// returns these codes where the reference would call exit().
enum Status : int {
    kOk = 0,
    kErrCuda = 1,
    kErrArg = 2,
    kErrNotInit = 3,
    kErrWeights = 4,
    kErrSingular = 5,
    kErrUnsupported = 6,
    kErrDeviceTimeout = 7,
    kErrNonFinite = 8,
    kErrNoMem = 9,
};

void set_error(int code, const char *fmt, ...);
int last_error();
const char *last_message();

#define SBTE_CUDA(call)                                                     \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            ::sbte::set_error(::sbte::kErrCuda, "%s:%d %s: %s", __FILE__,   \
                              __LINE__, #call, cudaGetErrorString(e_));     \
            return ::sbte::kErrCuda;                                        \
        }                                                                   \
    } while (0)

// Device-side status word: kernels record failures here instead of
// trapping.  Bit layout: bit 0 = a bounded wait gave up, bit 1 = a
// non-finite value was seen.
struct DeviceStatus {
    unsigned int flags;
    unsigned int where;
};

constexpr unsigned kStatusTimeout = 1u;
constexpr unsigned kStatusNonFinite = 2u;

__host__ __device__ inline int cdiv(int a, int b) { return (a + b - 1) / b; }

}  // namespace sbte
