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
// 1 when the network runs in its equilibrium-exact form (fno.cu header).
int fno_equilibrium(const spectral_fno_s *net);
// out[0] = sum of the squares of n FP64 device values (device double).
int batch_sumsq(const double *A, long long n, double *out, cudaStream_t st);
// out[0] = |A - R| / sqrt(|R|^2 + eps * msq[0] / B) for one instance of n3
// values: the spot check's relative distance with a floor of eps times the
// batch's mean squared instance norm (msq from batch_sumsq over B instances).
int rel_l2_floor_device(const double *A, const double *R, long long n3, const double *msq,
                        double eps, int B, double *out, cudaStream_t st);

}  // namespace sbte
