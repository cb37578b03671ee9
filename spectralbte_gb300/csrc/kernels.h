// kernels.h -- launchers shared between the CUDA translation units of the
// library.  All launchers are asynchronous on the given stream and return a
// cudaError_t from the launch (not from execution).
#pragma once

#include <cuda_runtime.h>

namespace sbte {

// ---------------------------------------------------------------- DFT ---
// The phase-shifted 3D transform of the reference's fft3D
// (collisions.c:232-283), as three dense N x N axis matrices:
//   out = prefactor * (D (x) D (x) D) in,
//   D[k][n] = exp(i s L_end varr[k]) exp(i dir 2 pi (n k mod N)/N) wt[n]
//             exp(i s n L_start delta).
// Dt holds D transposed (Dt[n*N + k] = D[k][n]) in the compute precision.
//
// Batched layouts: element (b, pos) of an array with group width bg sits at
//   (b / bg) * (N^3 * bg) + pos * bg + (b % bg)
// bg = 1 is the plain instance-major layout [b][pos].

enum class DftIn { kRealF64, kComplexF64, kComplexF32 };
// kF4 / kG4: FP32 complex z written as the packed operand quadruples of
// the expanded-operand convolution, (z.x, z.y, z.y, z.x) and
// (z.x, z.x, -z.y, z.y).
enum class DftOut { kComplexF64, kComplexF32, kRealF64, kRealF32, kF4, kG4 };

// Forward or inverse 3D DFT of B instances, FP64 arithmetic.
// in: real or complex FP64; tmp: B*N^3 double2 scratch; out: complex FP64
// (kComplexF64) or its real part (kRealF64).
cudaError_t dft3_f64(const void *in, DftIn in_kind, int in_bg, double2 *tmp,
                     void *out, DftOut out_kind, int out_bg,
                     const double2 *Dt, double prefactor, int N, int B,
                     cudaStream_t st);

// Same in FP32 arithmetic; in may be real FP64 (f from the caller) or
// complex FP32; out complex FP32 or real FP64/FP32.
cudaError_t dft3_f32(const void *in, DftIn in_kind, int in_bg, float2 *tmp,
                     void *out, DftOut out_kind, int out_bg,
                     const float2 *Dt, float prefactor, int N, int B,
                     cudaStream_t st);

// ------------------------------------------------------- convolution ---
// qhat[b][zeta] = sum_xi W[zeta][xi] * P_b[xi] * R_b[idx(zeta, xi)]
//               (+ S_b[xi] * T_b[idx(zeta, xi)] when S != nullptr),
// idx per axis = (zeta_a + N/2 - xi_a) wrapped once into [0, N)
// (collisions.c:141-160).  W is row-major [N^3][N^3] FP64.  All complex
// arrays use the plain layout [b][pos].  qhat is written, not accumulated.
cudaError_t conv_f64(const double *W, const double2 *P, const double2 *R,
                     const double2 *S, const double2 *T, double2 *qhat,
                     int N, int B, cudaStream_t st);

// The FP32 batched convolution.  Wblk is FP32 in the tiled layout
// [zrow][xrow][zz][xz] (zrow = zx*N+zy, xrow = xx*N+xy); P,R,S,T are
// complex FP32 in the bg-interleaved layout; qacc is a FP64 accumulator in
// the same interleaved layout [group][zeta][bg] (re, im); status receives
// the bounded-wait flags.  Returns cudaErrorInvalidValue for unsupported
// (N, bg).
struct ConvF32Config {
    int bg;           // instances per CTA (32, 64 or 128)
    int stages;       // copy pipeline depth (variant 1: 2 or 3)
    int flush;        // xi-rows between FP64 flushes of the FP32 partial sums
    int variant = 1;  // 1: block-barrier kernel; 2: warp-specialised with
                      // packed FP32x2 math; 3: warp-specialised, scalar math;
                      // 4: warp-specialised, FP32x2 on expanded operands;
                      // 5: as 3, registers capped for 2 CTAs per SM
    int zs = 0;       // variants 2, 3: zeta_z values per thread (8 or 16)
    int sym = 0;      // variants 2, 3, 5: symmetric form over partner xi-rows
                      // (Wblk is then the table of weights_to_sym_f32)
    // Test hook of the bounded waits (variants 2, 3, 5): with stall_slot >= 0
    // the first CTA's producer skips that slot's copies and the CTA's waits
    // give up after stall_limit clocks (conv_ws.cu).
    int stall_slot = -1;
    long long stall_limit = 0;
};
cudaError_t conv_f32_batched(const float *Wblk, const float2 *P,
                             const float2 *R, const float2 *S,
                             const float2 *T, double2 *qacc, int N, int B,
                             ConvF32Config cfg, unsigned int *status,
                             cudaStream_t st);
size_t conv_f32_smem_bytes(int N, ConvF32Config cfg, bool two_pairs);
bool conv_f32_supported(int N, ConvF32Config cfg, bool two_pairs);

// The warp-specialised FP32x2 variant (conv_ws.cu); writes qacc on its
// first flush, so it needs no zeroed accumulator.
// minb: CTAs per SM the kernel's register budget is sized for (1, or 2 for
// variant 5).
bool conv_ws_supported(int N, int bg, int zs, bool packed, int stages,
                       bool two_pairs, int minb);
cudaError_t conv_ws(const float *Wblk, const float2 *P, const float2 *R,
                    const float2 *S, const float2 *T, double2 *qacc, int N, int B,
                    int bg, int zs, bool packed, int stages, int flush, int sym,
                    int minb, unsigned int *status, cudaStream_t st,
                    int stall_slot = -1, long long stall_limit = 0);

// Symmetric form of the convolution for g = f (both Q(f,f) and the
// maxPreserve sum).  For zeta-row (zx, zy) the xi-row partner map is
// r = (xx, xy) -> (sx, sy), s_a = (z_a + N/2 - x_a) mod N; a row is run
// when its partner does not precede it (flat index sx*N+sy >= xx*N+xy).
// For even N an axis has two self-partnered values when z_a + N/2 is even
// and none otherwise, so a zeta-row runs N^2/2 + 2 slots when both axes
// have them and N^2/2 otherwise.
__host__ __device__ inline int sym_slots(int N, int zx, int zy)
{
    const int h = N / 2;
    return (N * N) / 2 + ((((zx + h) & 1) == 0 && ((zy + h) & 1) == 0) ? 2 : 0);
}
__host__ __device__ inline int sym_max_slots(int N) { return (N * N) / 2 + 2; }
// Wsym[zrow][slot][zz][xz] (FP32) for the slots in run order: the tile of
// row r plus, when r is not its own partner, the partner's tile with xz
// mapped through s_z = (zz + N/2 - xz) mod N, summed in FP64.  Slots beyond
// sym_slots of a zeta-row are zero.  N even; size N^2 * sym_max_slots * N^2.
cudaError_t weights_to_sym_f32(const double *W, float *Wsym, int N, cudaStream_t st);

// The expanded-operand FP32x2 convolution (variant 4): W tiled with every
// value as a (w, w) pair; P, S in the G4 form and R, T in the F4 form
// (DftOut), all bg-interleaved.
bool conv_x4_supported(int N, int bg, int zs, int stages, bool two_pairs);
cudaError_t conv_x4(const float2 *W2blk, const float4 *P, const float4 *R,
                    const float4 *S, const float4 *T, double2 *qacc, int N, int B,
                    int bg, int zs, int stages, int flush, unsigned int *status,
                    cudaStream_t st);
cudaError_t weights_to_tiled_f32x2(const double *W, float2 *W2blk, int N,
                                   cudaStream_t st);

// Re-layout of FP64 row-major W into the FP32 tiled layout.
cudaError_t weights_to_tiled_f32(const double *W, float *Wblk, int N,
                                 cudaStream_t st);

// --------------------------------------------- moments / conservation ---
struct ConsParams {
    int N, Ns;
    double dv;
    double mass[4];
    double CCt[8][8];  // LU factors of CC^T (conserve.c:89-168)
    int pivot[8];
};
// Conservation projection (conserve.c:207-264) for one species on B
// independent instances Q[b][pos] (plain layout), in place, FP64.  A
// non-finite moment sum or multiplier sets kStatusNonFinite in *status
// (when status is not null).
cudaError_t conserve_batch(double *Q, int B, const double *v,
                           const ConsParams &cp, cudaStream_t st,
                           unsigned int *status = nullptr);
// Multi-species form: Qptrs[n*Ns+m] point at N^3 arrays (one instance).
cudaError_t conserve_species(double **Qptrs_dev, const double *v,
                             const ConsParams &cp, cudaStream_t st,
                             unsigned int *status = nullptr);

// Maxwellian split of find_maxwellians (collisions.c:91-106) for B
// instances: M = Maxwellian with the (rho, u, T) of f, computed with the
// momentRoutines.c formulas (mass, KB); g = f - Mref where Mref = M of the
// instance's "first" argument (the reference always subtracts M_i).
// When Mref == nullptr, g = f - M; when g == nullptr, only M is written.
cudaError_t maxwellian_split(const double *f, double *M, double *g,
                             const double *Mref, int B, int N,
                             const double *v, double mass, double KB,
                             double *moments_out, cudaStream_t st,
                             unsigned int *status = nullptr);

// Output moments of B instances, 8 doubles each: rho, u_x, u_y, u_z, T,
// rho T, and the positive and negative parts of getEnergy
// (output.c:156-213, momentRoutines.c:58-190).
cudaError_t moments_batch(const double *f, int B, int N, const double *v, double mass,
                          double KB, double *out, cudaStream_t st,
                          unsigned int *status = nullptr);

// Euler / RK2 combinations of boltz.c:206-241 on B*N^3 values.
cudaError_t axpy_update(double *y, const double *x, const double *q,
                        double a_y, double a_x, double a_q, long long n,
                        cudaStream_t st);

// ---------------------------------------------------------- transport ---
// The 1D-3V transport of transportroutines.c on one device array of
// nX + 2*order cells of N^3 values, for one rank.
struct TransportParams {
    int N, nX, order, ic;   // ic: the reference's Init_field (boundary kind)
    double dt, T0, T1, TWall, mass, KB;
};
// Ghost cells of upwindOne (walls, outflow copy or periodic).
cudaError_t transport_ghosts1(double *f, const double *v, const TransportParams &tp,
                              cudaStream_t st);
// upwindOne for cells 1..nX: fc from f (ghosts already set).
cudaError_t transport_upwind1(const double *f, double *fc, const double *v,
                              const double *dx, const TransportParams &tp,
                              cudaStream_t st);
// upwindTwo for cells 2..nX+1 (fills f's ghosts, wall values f_l, f_r).
cudaError_t transport_upwind2(double *f, double *fc, double *f_l, double *f_r,
                              const double *v, const double *x, const double *dx,
                              const TransportParams &tp, cudaStream_t st);

// ------------------------------------------------------------ weights ---
struct WeightParams {
    int N;
    double L_v, lambda, mu, dfac, prefactor;
    double zmax;  // max |zeta_a| over the grid
    // closed form: a gain argument below ztol is a zero of exact arithmetic
    // left by rounding (xi = mu zeta up to the last bit) and is taken as 0
    double ztol = 0.0;
};
// Largest panel count the row kernel supports (16 nodes per panel).
constexpr int kWeightMaxPanels = 160;
// Panels needed for the gain integral of the worst row of this grid.
int weights_panels_needed(const WeightParams &wp);
// Isotropic weights (weights.c:265-281), FP64, rows [row0, row0+nrows),
// row-major into W.  zeta is the device Fourier grid.
cudaError_t weights_iso(double *W, int row0, int nrows, const double *zeta,
                        const WeightParams &wp, const double *glx,
                        const double *glw, double *loss_scratch,
                        cudaStream_t st);

// Landau weights (aniso_weights.c:370-425) for rows [row0, row0 + nrows)
// into W[row - row0][N^3] (FP64); glx, glw: the 64-point Gauss-Legendre rule
// on [-1, 1] (device).
// Isotropic weights with the closed-form radial integral (lambda 0 or 1;
// weights.cu): FP64 rows [row0, row0 + nrows), or the row-pair FP32 table of
// the convolution (the layout of weights_to_sym_f32) with no FP64 table.
cudaError_t weights_iso_closed(double *W, int row0, int nrows, const double *zeta,
                               const WeightParams &wp, cudaStream_t st);
cudaError_t weights_sym_closed(float *Wsym, const double *zeta, const WeightParams &wp,
                               cudaStream_t st);
// Grazing-collision weights (MPIcollisionRoutines.c:33-205), one value per
// (zeta, xi) pair of pairs[6 u ..]: npan 16-point panels in r and phi, the
// nte theta panels between te[0..nte]; glx, glw the 16-point rule.
cudaError_t weights_graze(double *vals, const double *pairs, int npairs, double L_v,
                          double lambda, double glance, int npan, const double *te, int nte,
                          const double *glx, const double *glw, cudaStream_t st);
// W[e] = vals[map[e]], e < n.
cudaError_t weights_scatter(double *W, const double *vals, const int *map, long long n,
                            cudaStream_t st);
cudaError_t weights_landau(double *W, int row0, int nrows, const double *zeta, int N,
                           double L_v, double lambda, const double *glx, const double *glw,
                           cudaStream_t st);

}  // namespace sbte
