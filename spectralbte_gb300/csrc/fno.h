// fno.h -- internal interface of the learned collision operator (fno.cu)
// for the plan code in capi.cu.
#pragma once

#include <cuda_runtime.h>

struct spectral_fno_s;

namespace sbte {

// Network output for B instances: Q[b][pos] (FP64, plain layout) from
// f[b][pos] (FP64), before any conservation projection.
int fno_predict(spectral_fno_s *net, const double *f, double *Q, int B, cudaStream_t st);
int fno_grid_n(const spectral_fno_s *net);
// Allocate the inference buffers for B instances now (before a graph capture).
int fno_reserve(spectral_fno_s *net, int B);
// Relative L2 distance of instance b of A from instance b of Bref, each
// [*][n3] FP64 on the device, written to out (device double).
int rel_l2_device(const double *A, const double *Bref, long long n3, double *out,
                  cudaStream_t st);
// Add n kernel launches to the library's launch counter.
void add_launches(int n);

}  // namespace sbte
