/*
 * spectral_bte.h -- C ABI of the GB300 spectral-Lagrangian collision library
 * (libspectral_gb300.so).
 *
 * Part 1 exports the reference's own collision-path symbols with identical
 * signatures.  The reference's C host (boltz.c, initializer.c, output.c,
 * transportroutines.c, ...) links against this library instead of
 * collisions.c, conserve.c and weights.c, and runs unchanged.  Each
 * declaration cites the reference declaration it replaces.
 *
 * Part 2 adds batched entry points that keep f, fhat and Q resident in
 * device memory.  They replace the caller-side loop over cells
 * (boltz.c:285-345) and over independent 0D instances.
 *
 * Conventions kept from the reference:
 *   - index (i,j,k) -> k + N*(j + N*i), i slowest (collisions.c:99-102);
 *   - W is N^3 rows (zeta) of N^3 columns (xi), FP64 (weights.c:61-63);
 *   - Weights/ cache files are raw native-endian float64, N^3 rows x N^3,
 *     no header, named as in weights.c:68,70,73.
 * Errors: the reference's entry points return void and exit() on failure.
 * Here they record a status that spectral_last_error() returns and print
 * one line to stderr.  They never exit and never trap on the device.
 */
#ifndef SPECTRAL_BTE_H
#define SPECTRAL_BTE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* fftw_complex layout (interleaved re, im), without FFTW. */
#if !defined(FFTW3_H) && !defined(ORACLE_STUB_FFTW3_H) && !defined(SPECTRAL_HAVE_FFTW_COMPLEX)
#define SPECTRAL_HAVE_FFTW_COMPLEX
typedef double fftw_complex[2];
#endif

/* Layout-compatible with the reference's species (species.h:11-26); same
   include guard so the two headers coexist. */
#ifndef _SPECIES_H
#define _SPECIES_H
typedef struct {
    size_t id;
    size_t num_levels;
    size_t *lev_id;
    double Rgas;
    double mass;
    double mm;
    double d_ref;
    double T_ref;
    double mu_ref;
    double omega;
    double E0;
    double *Ei;
    double *gi;
    char name[80];
} species;
#endif

/* ===================== Part 1: reference symbols ====================== */

/* collisions.h:27 (defined collisions.c:33) */
void initialize_coll(int nodes, double length, double *vel, double *zeta);
/* collisions.h:33 (collisions.c:81) */
void dealloc_coll(void);
/* collisions.h:38 (collisions.c:212): Q = Re(IFFT(Qhat(f, g))), FP64 */
void ComputeQ(double *f, double *g, double *Q, double **conv_weights);
/* collisions.h:40 (collisions.c:178): Q(M_i,g_j) + Q(g_i,M_j) + Q(g_i,g_j) */
void ComputeQ_maxPreserve(double *f, double *g, double *Q,
                          double **conv_weights);
/* collisions.h:42 (collisions.c:232) */
void fft3D(fftw_complex *in, fftw_complex *out, int invert);

/* conserve.h:6 (conserve.c:17) */
void initialize_conservation(int nodes, double h_v, double *vel, species *mix,
                             int num_spec);
/* conserve.h:8 (conserve.c:45) */
void initialize_conservation_fast(int nodes, double h_v, double *vel);
/* conserve.h:10 (conserve.c:76) */
void dealloc_conservation(void);
/* conserve.h:12 (conserve.c:89); det is unused, as in the reference */
void factorMatrixIntoLU(int nElem, double det);
/* conserve.h:14 (conserve.c:173) */
void solveWithCCt(int nElem, double *b);
/* conserve.h:16 (conserve.c:207) */
void conserveAllMoments(double **Q);
/* conserve.h:18 (conserve.c:268) */
void createCCtAndPivot(void);

/* weights.h:12 (weights.c:26) */
void alloc_weights(int N, double ****conv_weights, int total_species);
/* weights.h:37 (weights.c:33): load Weights/<name>.wts or generate it on
   the GPU and store it; also keeps a device copy keyed by conv_weights */
void initialize_weights(int nodes, double *eta, double Lv, double lam,
                        int weightFlag, int isoFlag, double **conv_weights,
                        species species_i, species species_j);
/* weights.h:45 (weights.c:127) */
/* aniso_weights.c:37 (definition order; aniso_weights.h:1 swaps Lv and lam,
   and boltz.c:154 calls it in definition order).  Loads
   Weights/N%d_Aniso_L_v%g_lambda%g_Landau.wts (glance = 0) or
   Weights/N%d_AnIso_L_v%g_lambda%g_glance%g.wts (glance != 0), or generates
   the weights on the GPU and writes that file.  The weights are the Landau
   kernel for every glance, as in the reference: its generator branches on a
   file-scope glance (aniso_weights.c:31,417) that the parameter shadows and
   nothing sets. */
void initialize_weights_AnIso(int nodes, double *zeta, double Lv, double lam,
                              int weightFlag, double **conv_weights,
                              double glance);
void dealloc_weights(int N, double **conv_weights);
/* exec/MPIWeightGenerator.c (the `weights_ N glance beta lambda L_v`
   executable, main :37-127): on its own grid (:63-74), Landau weights for
   glance = 0 or grazing-collision weights otherwise, written to
   Weights/N%d_Aniso_L_v%g_lambda%g_Landau.wts or
   Weights/N%d_AnIso_L_v%g_lambda%g_glance%g.wts (:79-83) unless the file
   exists; initialize_weights_AnIso with the same arguments then loads it.
   One GPU replaces the MPI ranks; beta is unused, as in the reference.
   Returns a status (the reference exits). */
int spectral_weights_generator(int N, double glance, double beta, double lambda,
                               double L_v);
/* weights.h:43 (weights.c:265): GPU quadrature into conv_weights rows */
void generate_conv_weights_iso(double **conv_weights);
/* weights.h:47 (weights.c:156): the integrand, on the host */
double ghat(double r, void *args);
/* weights.h:49 (weights.c:181): one weight's integral times prefactor */
double gHat3(double ki1, double ki2, double ki3, double zeta1, double zeta2,
             double zeta3);

/* ===================== Part 2: batched device API ===================== */

/* Status codes (returned by spectral_* and spectral_last_error). */
#define SPECTRAL_OK 0
#define SPECTRAL_ERR_CUDA 1
#define SPECTRAL_ERR_ARG 2
#define SPECTRAL_ERR_NOT_INIT 3
#define SPECTRAL_ERR_WEIGHTS 4
#define SPECTRAL_ERR_SINGULAR 5
#define SPECTRAL_ERR_UNSUPPORTED 6
#define SPECTRAL_ERR_DEVICE_TIMEOUT 7
#define SPECTRAL_ERR_NONFINITE 8
#define SPECTRAL_ERR_NOMEM 9

/* Flags for spectral_computeQ_*. */
#define SPECTRAL_FP64 0        /* plain FP64 operator (parity path) */
#define SPECTRAL_FP32 1        /* batched FP32 convolution + FFTs */
#define SPECTRAL_MAXPRESERVE 2 /* ComputeQ_maxPreserve semantics */
#define SPECTRAL_CONSERVE 4    /* apply conserveAllMoments (FP64) */
#define SPECTRAL_LEARNED 8     /* learned operator + spot check (see below) */

int spectral_last_error(void);
const char *spectral_last_error_message(void);
const char *spectral_version(void);

typedef struct spectral_plan_s spectral_plan;

/* A plan holds one velocity grid (N nodes on [-L_v, L_v]; v and zeta as
   the reference's initializer builds them), its device weights, the
   conservation factors for one species and scratch for up to max_batch
   instances.  It uses the CUDA device current at creation. */
int spectral_plan_create(spectral_plan **plan, int N, double L_v,
                         const double *v, const double *zeta, int max_batch);
int spectral_plan_destroy(spectral_plan *plan);

/* Weights: from host rows (reference layout), from one flat row-major
   [N^3][N^3] array (host or device), or generated on the GPU by the
   isotropic quadrature (weights.c:265-281).  Species diameters and masses
   as species.c defaults: d = 2, m = 1. */
int spectral_plan_set_weights_rows(spectral_plan *plan, double **rows);
int spectral_plan_set_weights(spectral_plan *plan, const double *W,
                              int on_device);
int spectral_plan_generate_weights_iso(spectral_plan *plan, double lambda,
                                       double d_i, double d_j, double m_i,
                                       double m_j);
int spectral_plan_get_weights(spectral_plan *plan, double *W_host,
                              long long row0, long long nrows);
/* Conservation factors for one species of the given mass
   (initialize_conservation with Ns = 1). */
/* Landau weights (aniso_weights.c:370-425: the 64 x 64-point Gauss-Legendre
   double integral of gHat3L, no trapezoid factors) for the plan's grid. */
int spectral_plan_generate_weights_landau(spectral_plan *plan, double lambda);
int spectral_plan_set_conservation(spectral_plan *plan, double mass);
/* Isotropic weights with the radial integral of weights.c:156-160 in closed
   form (lambda 0 or 1 only; the quadrature covers every lambda): the same
   table as spectral_plan_generate_weights_iso to ~1e-14, in a fraction of
   the time.  fp64_table = 1 stores the FP64 table as usual.  fp64_table = 0
   builds only the row-pair FP32 table of the convolution, directly from the
   closed form, and never holds the FP64 table (8 N^6 bytes: 8.6 GB at
   N = 32, 98 GB at N = 48): the plan then serves SPECTRAL_FP32 calls only
   (FP64 calls and spectral_plan_get_weights return SPECTRAL_ERR_WEIGHTS), in
   the row-pair form, and supports N = 48.  The reference's commented-out
   closed form (weights.c:216-253) and its unimplemented weightgen option
   (boltz.c:56,162-164) point at this. */
int spectral_plan_generate_weights_closed(spectral_plan *plan, double lambda,
                                          double d_i, double d_j, double m_i,
                                          double m_j, int fp64_table);
/* Grazing-collision weights: gHat3 of the stand-alone generator
   (MPIcollisionRoutines.c:33-205, eps-linear cross section with the
   Coulomb-case Taylor term below theta = sqrt(glance)), no trapezoid
   factors, for the plan's grid; 0 < glance < pi^2/4, N <= 16.  The
   reference's GSL QAG/CQUAD (tolerance 1e-6) is replaced by composite
   Gauss-Legendre rules converged to ~1e-13. */
int spectral_plan_generate_weights_grazing(spectral_plan *plan, double lambda,
                                           double glance);

/* Q for B instances.  f and Q are [B][N^3] FP64 in device memory; for
   flag SPECTRAL_FP32 the transforms and the convolution run in FP32 and
   moments, Maxwellian split and conservation stay FP64.  stream is a
   cudaStream_t; NULL is the default stream, as in the CUDA runtime.
   Asynchronous with respect to the host. */
int spectral_computeQ_device(spectral_plan *plan, const double *f_dev,
                             double *Q_dev, int B, int flags, void *stream);
/* Same with host arrays: copies in, computes, copies out, synchronises.  The
   batch runs in chunks of whole instance groups on the plan's stream, with
   the copies on two other streams, so that each chunk's copies overlap the
   neighbouring chunks' compute (pinned host memory makes the copies
   asynchronous). */
int spectral_computeQ_host(spectral_plan *plan, const double *f_host,
                           double *Q_host, int B, int flags);
/* conserveAllMoments on [B][N^3] device arrays, FP64, in place. */
int spectral_conserve_device(spectral_plan *plan, double *Q_dev, int B,
                             void *stream);
/* One time step of the homogeneous solver (boltz.c:193-241) for B
   instances held on the device: order 1 (Euler) or 2 (RK2), f updated in
   place.  Conservation is always applied, as boltz.c does. */
int spectral_step_device(spectral_plan *plan, double *f_dev, int B,
                         double dt, double Kn, int order, int flags,
                         void *stream);

/* Uneven batches: Q for several plans at once (one plan per velocity grid
   N and weight table, e.g. N in {16, 24, 32} x lambda in {0, 1}).  Plan i
   evaluates B[i] instances f_dev[i] -> Q_dev[i] on its own stream, forked
   from and joined back to `stream`, so the groups overlap on the device. */
int spectral_group_computeQ(spectral_plan **plans, int nplans,
                            const double *const *f_dev, double *const *Q_dev,
                            const int *B, int flags, void *stream);

/* 1D-3V solver on the device (boltz.c:264-394 for one species, one rank).
   f holds nX + 2*order cells of N^3 values, interior cells order ..
   nX+order-1; x and dx hold the cell centres and widths of all of them
   (the reference's make_mesh layout).  ic is the reference's Init_field,
   which selects the boundaries: 3 and 5 diffuse walls at T0 (left) and T1
   (right), 1 a heated left wall at 2*TWall, 6 periodic, others outflow.
   Transport is upwindOne (order 1) or the minmod advectTwo (order 2);
   collisions run for all nX cells in one batched call with conservation,
   then Euler (order 1) or RK2 (order 2), exactly as boltz.c orders them. */
int spectral_1d_setup(spectral_plan *plan, int nX, int order, int ic, double dt,
                      double Kn, const double *x, const double *dx, double T0,
                      double T1, double TWall, double mass);
int spectral_1d_step(spectral_plan *plan, double *f_dev, int flags, void *stream);
/* The transport alone: fconv = advect(f) (also fills f's ghost cells). */
int spectral_1d_advect(spectral_plan *plan, double *f_dev, double *fconv_dev,
                       void *stream);

/* CUDA graph of one time step: kind 0 = spectral_step_device(f, B, dt,
   Kn, order, flags), kind 1 = spectral_1d_step(f, flags).  All scratch is
   allocated before the capture; the graph replays on f_dev. */
int spectral_graph_capture(spectral_plan *plan, int kind, double *f_dev, int B,
                           double dt, double Kn, int order, int flags);
int spectral_graph_launch(spectral_plan *plan, void *stream);

/* FP32 convolution tuning.  variant 1 = block-barrier kernel; 2 = warp-
   specialised kernel with packed FP32x2 math; 3 = warp-specialised, scalar
   math; 4 = warp-specialised, FP32x2 on pre-expanded operands; 5 = as 3 with
   the registers capped so that two CTAs of 64 instances (or three of 32)
   share an SM (one-pair form only: maxPreserve calls run variant 3's shape
   instead).  A call of at most 32 instances runs the plan's shape with a
   group of 32 where one exists; the result is the same bit for bit.
   bg = instances per CTA (32, 64, 128); zs = zeta_z values per thread
   (variants 2-5: 8 or 16);
   stages = copy pipeline depth; flush = xi-rows per FP64 flush.  Shapes
   that are not instantiated return SPECTRAL_ERR_UNSUPPORTED.  The
   autotuner times the supported shapes on B instances and keeps the
   fastest; *chosen (optional, 5 ints: variant, bg, zs, stages, flush)
   receives it. */
int spectral_plan_set_tuning(spectral_plan *plan, int variant, int bg, int zs,
                             int stages, int flush);
int spectral_plan_autotune(spectral_plan *plan, int B, int flags,
                           int *chosen);
/* Symmetric form of the warp-specialised FP32 convolution (variants 2, 3;
   on by default).  Every FP32 call here has g = f, and for a fixed zeta the
   xi-rows r and (zeta + N/2 - r) mod N see the same product of transforms,
   so one pass over a row pair with the two weight tiles summed (in FP64,
   one rounding) replaces two: (N^2 + F)/2 of the N^2 rows per zeta-row
   (F = 0 or 4 self-paired rows).  The same sum in another order; off runs
   every row with the plain tiled weights. */
int spectral_plan_set_symmetric(spectral_plan *plan, int on);

/* Device status word of the calls since the last read: bit 0 = a bounded
   device wait gave up (the kernel then left early and its output is not
   valid), bit 1 = a non-finite moment sum (NaN or infinity in f or Q; set by
   the conservation, Maxwellian-split and moment kernels).  Cleared by the
   read.  No counterpart in the reference, which neither bounds its waits nor
   checks for NaN. */
int spectral_plan_status(spectral_plan *plan, unsigned int *status);
/* Test hook of the bounded waits, no counterpart in the reference.  The next
   FP32 convolution launch of the plan (warp-specialised variants 2, 3, 5)
   skips the copies of pipeline slot `slot` in its first CTA, whose waits then
   give up after limit_clocks (1e3 .. 2^31): that CTA's consumers wait on a
   barrier that nothing completes, set bit 0 of the status word and leave,
   and every other CTA runs normally.  One shot.  The call's result is not
   valid; the plan stays usable. */
int spectral_plan_inject_stall(spectral_plan *plan, int slot, long long limit_clocks);

/* Convolution-kernel timing: with profiling on, every convolution launch
   is bracketed by CUDA events on its own stream; spectral_plan_conv_time
   returns the summed device time (ms) and the number of launches since
   the last query, then resets. */
int spectral_plan_set_profiling(spectral_plan *plan, int on);
int spectral_plan_conv_time(spectral_plan *plan, double *total_ms,
                            int *launches);

/* Synchronise the plan's stream. */
int spectral_plan_sync(spectral_plan *plan);

/* Allocation-free batched 3D transform.  No counterpart in the reference:
   it is fft3D (forward for invert = 0, inverse otherwise) on B instances of
   interleaved complex [B][N^3] device arrays, for callers that cannot call
   cudaMalloc, e.g. a solver inside a host application that owns all device
   memory through its own pool, or a step in a time-critical loop.  It
   allocates nothing.  Its scratch (the axis matrix and the plane-pass
   intermediate) is one static 32 MiB device array that every GPU loading
   the library holds until exit; N^2 + B*N^3 must not exceed 2,097,152
   complex values (N = 32: B <= 63), larger sizes return SPECTRAL_ERR_ARG.
   The first call on a device looks up the array's device address, so make
   it before any stream capture.  Under CUDA's lazy module loading (the
   default since CUDA 12.2) the array comes into being when the library's
   device code first loads on that device, which may be at that first call:
   the call then takes the 32 MiB from device memory, so a host that pools
   all device memory makes its first call before the pool takes it.  All calls share the array and nothing in
   it needs to start at zero; calls that overlap on the GPU race.  in_dev
   may equal out_dev.  Asynchronous on stream (NULL: default stream). */
int spectral_fft3d_noalloc(int N, double L_v, const double *v,
                           const double *zeta, const double *in_dev,
                           double *out_dev, int B, int invert, void *stream);

/* Output moments of B instances f_dev[B][N^3] (device) into out_dev[B][8]
   (device): rho, u_x, u_y, u_z, T, rho T, and the positive and negative
   parts of getEnergy -- everything write_streams / write_streams_inhom print
   (output.c:156-213,295-404), so a dump reads 64 bytes per cell instead of
   f.  Uses the plan's mass and KB.  Asynchronous on stream. */
int spectral_moments_device(spectral_plan *plan, const double *f_dev, int B,
                            double *out_dev, void *stream);

/* ---- Learned collision operator.  No counterpart in the reference.
   A Fourier neural operator maps f (one instance on the N^3 grid) to Q(f):
   lift to `width` channels, `layers` spectral layers on the lowest
   `modes`^3 Fourier modes (weights shared by modes of equal |m|^2) plus a
   pointwise channel mix and GELU, then a two-layer pointwise projection
   with `hidden` channels.  kind 0 applies GELU after every spectral layer
   but the last and reads out y = q2 . gelu(u) + c2; kind 1 keeps the layers
   linear and reads out the quadratic form y = c2 + sum_e q2[e] u_l(e) u_r(e)
   over hidden/2 channel pairs (rows 16 (e/8) + e%8 and that + 8), the form
   of a separable approximation of the collision kernel.  f is scaled by its
   maximum s and the output by s^2 times the output scale (Q is bilinear in
   f).  All GEMMs run on 16-bit tensor cores with FP32 accumulation:
   precision 0 stores activations and GEMM operands as BF16, precision 1 as
   FP16 (same rate, 3 more mantissa bits; the backward pass then carries a
   loss scale).  Parameters are FP32.  Shapes: N 4..32, width 8..64
   (multiple of 8), even modes <= min(16, N), layers 1..8, hidden 16..128
   (multiple of 16). */
typedef struct spectral_fno_s spectral_fno;
int spectral_fno_create(spectral_fno **net, int N, int width, int modes,
                        int layers, int hidden, int kind, int precision,
                        unsigned long long seed);
int spectral_fno_precision(spectral_fno *net);
/* Channel-mix timing: with profiling on, CUDA events are recorded on the
   launching stream around every channel-mix launch (the separate-kernel
   path, outside graph captures); spectral_fno_kernel_time returns their
   summed duration and count since profiling was switched on. */
int spectral_fno_set_profiling(spectral_fno *net, int on);
int spectral_fno_kernel_time(spectral_fno *net, double *ms_total, int *launches);
/* Channel-mix kernel of inference passes (default 4, the fastest on GB300:
   3.15 ms per layer at N = 32 and 1,024 instances against 5.36 ms for the
   general GEMM): 1 runs the
   warp-specialised kernel that moves its tiles with the tensor memory
   accelerator (2D cp.async.bulk.tensor loads and stores, mbarrier ring) where
   the shape allows (width 64, instances padded to a multiple of 64), with 4
   consumer warps, 3 stages, 3 CTAs per SM; 2 the same with 8 consumer warps
   and 2 CTAs per SM; 3 with 4 stages and 2 CTAs per SM; 4 with 8 consumer
   warps, 2 stages and 3 CTAs per SM; 5 with 16 consumer warps and 2 CTAs per
   SM; 6 as 4 with one staging tile per warp and 4 CTAs per SM; 0 runs the
   general tensor-core GEMM.  All give the same result. */
int spectral_fno_set_channel_mix_kernel(spectral_fno *net, int tma);
/* Readout kernel of inference passes: 1 (default) runs the warp-specialised
   TMA kernel where the shape allows (kind 0, width 64, hidden 128, instances
   padded to a multiple of 64); 0 the general GEMM.  The two sum the hidden
   rows in a different order: the outputs agree to FP32 rounding. */
int spectral_fno_set_readout_kernel(spectral_fno *net, int tma);
/* Axis-k transforms of inference passes (the first forward and the last
   inverse axis pass of every layer): 1 (default) runs the warp-specialised
   TMA kernel where the shape allows (N = 32, modes <= 16); 0 the general
   GEMM.  Same products, same K blocks: the same result. */
int spectral_fno_set_axis_kernel(spectral_fno *net, int tma);
/* Device status word of the network's kernels (bit 0: a bounded wait gave
   up); cleared by the read. */
int spectral_fno_status(spectral_fno *net, unsigned int *status);
int spectral_fno_destroy(spectral_fno *net);
long long spectral_fno_num_params(spectral_fno *net);
int spectral_fno_num_classes(spectral_fno *net);
/* Flat FP32 parameter vector: P, bP, then per layer W (width x width), b,
   R (classes x width x width), then Q1 (hidden x width), c1, q2 (hidden, or
   hidden/2 for kind 1), c2.
   set_params also resets the optimiser state. */
int spectral_fno_get_params(spectral_fno *net, float *host);
int spectral_fno_set_params(spectral_fno *net, const float *host);
int spectral_fno_set_output_scale(spectral_fno *net, float sigma);
float spectral_fno_output_scale(spectral_fno *net);
/* Network output Q[b][pos] (FP64 device) for f[b][pos], no projection. */
int spectral_fno_predict(spectral_fno *net, const double *f_dev, double *Q_dev,
                         int B, void *stream);
/* Loss floor eps >= 0 (default 0): the training loss of each instance is
   |y - Q~|^2 / (|Q~|^2 + eps * mean over the batch of |Q~|^2), so that
   near-equilibrium instances with |Q~| -> 0 do not dominate. */
int spectral_fno_set_loss_floor(spectral_fno *net, float eps);
/* Loss power 1 <= k <= 8 (default 1): the training loss becomes
   mean_b e_b^k, e_b the instance's loss above, so that each instance's
   gradient is weighted by k e_b^(k-1) and the worst instances of a batch count
   for more.  The gradient used (and returned by spectral_fno_loss_grad) is
   that of the loss divided by the batch mean of those weights, the plain
   loss's scale.  Plain form only (kErrArg with the equilibrium form on). */
int spectral_fno_set_loss_power(spectral_fno *net, float k);
/* Equilibrium-exact form (on = 1): the operator becomes
   Q(f) = s_f^2 sigma y(f / s_f) - s_M^2 sigma y(M_f / s_M), where M_f is the
   Maxwellian with the density, bulk velocity and temperature of f
   (momentRoutines.c:58-185 with unit mass and KB), so Q(M) = 0 holds
   identically.  v holds the N velocity nodes of the grid (needed for M_f).
   f and M_f run as one batch of 2B instances, so an evaluation costs twice
   the plain network.  Training (loss_grad, train_step) then fits the
   difference. */
int spectral_fno_set_equilibrium(spectral_fno *net, int on, const double *v);
int spectral_fno_equilibrium(spectral_fno *net);
/* Mean over instances of |y - Q~|^2 / |Q~|^2 (Q~ = Q / (s^2 sigma), with the
   loss floor above) and its gradient (host, nparams floats) for FP32 device
   data f, Q [B][N^3]. */
int spectral_fno_loss_grad(spectral_fno *net, const float *f_dev,
                           const float *Q_dev, int B, double *loss_out,
                           float *grad_host);
/* One Adam step (beta 0.9 / 0.999) on that loss; loss_out may be NULL
   (no host synchronisation then). */
int spectral_fno_train_step(spectral_fno *net, const float *f_dev,
                            const float *Q_dev, int B, float lr,
                            double *loss_out, void *stream);
/* Attach a network to a plan for computeQ with SPECTRAL_LEARNED: the
   network output is projected by the FP64 conservation step; every
   check_every-th call one instance is recomputed with the plain FP32
   operator, and a rel-L2 distance above tol switches to the plain operator
   (the other flags) until a later check passes.  check_every = 0 never
   checks.  net = NULL detaches. */
int spectral_plan_set_learned(spectral_plan *plan, spectral_fno *net,
                              double tol, int check_every);
/* Floor of the spot check (default 0): with eps > 0 the check's distance is
   |Q_net - Q| / sqrt(|Q|^2 + eps * mean over the batch of |Q_net,b|^2), the
   normalisation of the training loss with the same eps.  Near equilibrium
   Q -> 0, so the relative distance of any approximation with a given
   absolute error grows without bound; the floor measures the error against
   the collision term's scale in the batch instead. */
int spectral_plan_set_learned_floor(spectral_plan *plan, double eps);
int spectral_plan_learned_stats(spectral_plan *plan, long long *calls,
                                long long *checks, long long *fallbacks,
                                double *last_err);

/* Number of kernels the library launched since load (monotonic). */
long long spectral_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* SPECTRAL_BTE_H */
