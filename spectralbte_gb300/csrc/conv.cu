// conv.cu -- the weighted Fourier-space convolution of compute_Qhat
// (collisions.c:125-165):
//
//   qhat[zeta] = sum_xi W[zeta][xi] * ghat[xi] * fhat[idx(zeta, xi)],
//   idx_a = zeta_a + N/2 - xi_a, wrapped once into [0, N) per axis.
//
// Two implementations:
//  * conv_f64: the plain FP64 operator.  A warp owns one (zeta, instance)
//    pair and its lanes stride along the W row, so row reads are coalesced.
//    A shuffle tree finishes the sum.  On GB300 this path is bound by the
//    FP64 pipe (6 FP64 instructions per term).
//  * conv_f32_batched: a CTA owns one zeta-row (zx, zy; all zz) for a group
//    of bg instances.  For each of the N^2 xi-rows it stages the N x N W
//    tile once in shared memory, with the matching ghat and fhat rows of
//    every instance in the group.  A cp.async.bulk (TMA) + mbarrier pipeline
//    does the staging, stages-deep.  The tile then serves all instances:
//    threads read W as a broadcast, and each thread keeps a sliding window
//    of fhat in registers for its own instance.  The FP32 partial sums
//    go to an FP64 accumulator in global memory every `flush` xi-rows.  That
//    is the compensated accumulation: FP32 error grows only over
//    flush*N terms.
#include "common.cuh"
#include "kernels.h"
#include "mbarrier.cuh"

#include <cstdint>

namespace sbte {
namespace {

__device__ __forceinline__ int wrap1(int x, int N)
{
    // One conditional +-N, as collisions.c:145-158 (always sufficient).
    return x < 0 ? x + N : (x > N - 1 ? x - N : x);
}

template <bool TWO>
__global__ void __launch_bounds__(256)
conv_f64_kernel(const double *__restrict__ W, const double2 *__restrict__ P,
                const double2 *__restrict__ R, const double2 *__restrict__ S,
                const double2 *__restrict__ T, double2 *__restrict__ qhat,
                int N)
{
    const int lane = threadIdx.x & 31;
    const int nn = N * N;
    const long long n3 = (long long)nn * N;
    const long long zeta = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int b = blockIdx.y;
    if (zeta >= n3) return;
    const int zx = (int)(zeta / nn), zy = (int)((zeta / N) % N), zz = (int)(zeta % N);
    const int h = N / 2;
    const double *Wrow = W + zeta * n3;
    const double2 *Pb = P + (long long)b * n3;
    const double2 *Rb = R + (long long)b * n3;
    const double2 *Sb = TWO ? S + (long long)b * n3 : nullptr;
    const double2 *Tb = TWO ? T + (long long)b * n3 : nullptr;
    double ar = 0.0, ai = 0.0;
    for (int xx = 0; xx < N; xx++) {
        const int x = wrap1(zx + h - xx, N);
        const long long xoff = (long long)xx * nn;
        for (int j = lane; j < nn; j += 32) {
            const int xy = j / N, xz = j - xy * N;
            const int y = wrap1(zy + h - xy, N), z = wrap1(zz + h - xz, N);
            const long long xi = xoff + j;
            const long long idx = ((long long)x * N + y) * N + z;
            const double w = __ldg(Wrow + xi);
            const double2 p = Pb[xi], r = Rb[idx];
            double pr = p.x * r.x;
            pr = fma(-p.y, r.y, pr);
            double pi = p.x * r.y;
            pi = fma(p.y, r.x, pi);
            if (TWO) {
                const double2 s = Sb[xi], t = Tb[idx];
                pr = fma(s.x, t.x, pr);
                pr = fma(-s.y, t.y, pr);
                pi = fma(s.x, t.y, pi);
                pi = fma(s.y, t.x, pi);
            }
            ar = fma(w, pr, ar);
            ai = fma(w, pi, ai);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, o);
        ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (lane == 0) qhat[(long long)b * n3 + zeta] = make_double2(ar, ai);
}

// ------------------------------------------------------------ FP32 ----

template <int N, int BG, bool TWO>
struct F32Layout {
    static constexpr int kWBytes = N * N * 4;
    static constexpr int kRowBytes = N * BG * 8;
    static constexpr int kRows = TWO ? 4 : 2;
    static constexpr int kStageBytes = kWBytes + kRows * kRowBytes;
};

// ZS = zeta_z values per thread; threads per CTA = BG * (N / ZS).
template <int N, int BG, int ZS, int STAGES, bool TWO>
__global__ void __launch_bounds__(BG *(N / ZS))
conv_f32_kernel(const float *__restrict__ Wblk, const float2 *__restrict__ P,
                const float2 *__restrict__ R, const float2 *__restrict__ S,
                const float2 *__restrict__ T, double2 *__restrict__ qacc,
                int flush, unsigned int *__restrict__ status)
{
    using L = F32Layout<N, BG, TWO>;
    constexpr int NN = N * N;
    constexpr int H = N / 2;
    constexpr long long N3 = (long long)NN * N;
    static_assert(N % 8 == 0, "xi_z chunks of 8");
    static_assert(N % ZS == 0, "zeta_z split");

    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[STAGES];
    __shared__ int abort_flag;

    const int tid = threadIdx.x;
    const int b = tid % BG;          // instance within the group
    const int zq = tid / BG;         // zeta_z segment
    const int z0 = zq * ZS;
    const int zrow = blockIdx.x;     // zeta row = zx*N + zy
    const int zx = zrow / N, zy = zrow % N;
    const long long grp = blockIdx.y;

    const float *Wbase = Wblk + (long long)zrow * NN * NN;
    const float2 *Pg = P + grp * N3 * BG;
    const float2 *Rg = R + grp * N3 * BG;
    const float2 *Sg = TWO ? S + grp * N3 * BG : nullptr;
    const float2 *Tg = TWO ? T + grp * N3 * BG : nullptr;

    if (tid == 0) {
        for (int s = 0; s < STAGES; s++) mbar_init(&full[s], 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    auto issue = [&](int it) {
        const int s = it % STAGES;
        unsigned char *base = smem + s * L::kStageBytes;
        const int xx = it / N, xy = it % N;
        const int fx = (zx + H - xx) < 0 ? zx + H - xx + N
                       : (zx + H - xx > N - 1 ? zx + H - xx - N : zx + H - xx);
        const int fy = (zy + H - xy) < 0 ? zy + H - xy + N
                       : (zy + H - xy > N - 1 ? zy + H - xy - N : zy + H - xy);
        const long long prow = (long long)it * N * BG;              // xi row
        const long long rrow = ((long long)fx * N + fy) * N * BG;   // idx row
        mbar_expect_tx(&full[s], L::kStageBytes);
        bulk_g2s(base, Wbase + (long long)it * NN, L::kWBytes, &full[s]);
        bulk_g2s(base + L::kWBytes, Pg + prow, L::kRowBytes, &full[s]);
        bulk_g2s(base + L::kWBytes + L::kRowBytes, Rg + rrow, L::kRowBytes, &full[s]);
        if (TWO) {
            bulk_g2s(base + L::kWBytes + 2 * L::kRowBytes, Sg + prow, L::kRowBytes, &full[s]);
            bulk_g2s(base + L::kWBytes + 3 * L::kRowBytes, Tg + rrow, L::kRowBytes, &full[s]);
        }
    };

    if (tid == 0) {
        for (int it = 0; it < STAGES && it < NN; it++) issue(it);
    }

    float2 acc[ZS];
#pragma unroll
    for (int i = 0; i < ZS; i++) acc[i] = make_float2(0.f, 0.f);

    double2 *qrow = qacc + grp * N3 * BG + ((long long)zrow * N + z0) * BG + b;
    int since_flush = 0;

    auto do_flush = [&]() {
#pragma unroll
        for (int i = 0; i < ZS; i++) {
            double2 q = qrow[(long long)i * BG];
            q.x += (double)acc[i].x;
            q.y += (double)acc[i].y;
            qrow[(long long)i * BG] = q;
            acc[i] = make_float2(0.f, 0.f);
        }
    };

    for (int it = 0; it < NN; it++) {
        const int s = it % STAGES;
        const uint32_t parity = (uint32_t)((it / STAGES) & 1);
        if (!mbar_wait_bounded(&full[s], parity)) {
            atomicOr(status, kStatusTimeout);
            abort_flag = 1;
        }
        __syncthreads();
        if (abort_flag) break;

        const unsigned char *base = smem + s * L::kStageBytes;
        const float *Ws = reinterpret_cast<const float *>(base);
        const float2 *Gs = reinterpret_cast<const float2 *>(base + L::kWBytes);
        const float2 *Fs = reinterpret_cast<const float2 *>(base + L::kWBytes + L::kRowBytes);
        const float2 *Ss = reinterpret_cast<const float2 *>(base + L::kWBytes + 2 * L::kRowBytes);
        const float2 *Ts = reinterpret_cast<const float2 *>(base + L::kWBytes + 3 * L::kRowBytes);

#pragma unroll 1
        for (int c = 0; c < N / 8; c++) {
            float2 gw[8];
            float2 sw[TWO ? 8 : 1];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                gw[e] = Gs[(8 * c + e) * BG + b];
                if (TWO) sw[e] = Ss[(8 * c + e) * BG + b];
            }
            // window: fw[d] = F[(z0 + H - 8c - 7 + d) mod N], d in [0, ZS+7)
            float2 fw[ZS + 7];
            float2 tw[TWO ? ZS + 7 : 1];
            int zi = z0 + H - 8 * c - 7;
            zi = ((zi % N) + N) % N;
#pragma unroll
            for (int d = 0; d < ZS + 7; d++) {
                fw[d] = Fs[zi * BG + b];
                if (TWO) tw[d] = Ts[zi * BG + b];
                zi = (zi == N - 1) ? 0 : zi + 1;
            }
#pragma unroll
            for (int zl = 0; zl < ZS; zl++) {
                const float4 wa = *reinterpret_cast<const float4 *>(Ws + (z0 + zl) * N + 8 * c);
                const float4 wb = *reinterpret_cast<const float4 *>(Ws + (z0 + zl) * N + 8 * c + 4);
                const float w[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    // zeta_z = z0+zl, xi_z = 8c+e  ->  window slot zl - e + 7
                    const float2 f = fw[zl - e + 7];
                    const float2 g = gw[e];
                    float pr = g.x * f.x;
                    pr = fmaf(-g.y, f.y, pr);
                    float pi = g.x * f.y;
                    pi = fmaf(g.y, f.x, pi);
                    if (TWO) {
                        const float2 t = tw[zl - e + 7];
                        const float2 q = sw[e];
                        pr = fmaf(q.x, t.x, pr);
                        pr = fmaf(-q.y, t.y, pr);
                        pi = fmaf(q.x, t.y, pi);
                        pi = fmaf(q.y, t.x, pi);
                    }
                    acc[zl].x = fmaf(w[e], pr, acc[zl].x);
                    acc[zl].y = fmaf(w[e], pi, acc[zl].y);
                }
            }
        }
        __syncthreads();  // everyone is done with stage s
        if (tid == 0 && it + STAGES < NN) issue(it + STAGES);
        if (++since_flush == flush) {
            do_flush();
            since_flush = 0;
        }
    }

    if (abort_flag) {
        // Let copies already in flight land before the CTA leaves
        // (bounded again), so no bulk copy targets freed shared memory.
        if (tid == 0) {
            for (int s = 0; s < STAGES; s++) (void)mbar_wait_bounded(&full[s], 0);
        }
        __syncthreads();
        return;
    }
    if (since_flush) do_flush();
}

template <int N, int BG, int ZS, int STAGES, bool TWO>
cudaError_t launch_f32(const float *Wblk, const float2 *P, const float2 *R,
                       const float2 *S, const float2 *T, double2 *qacc, int B,
                       int flush, unsigned int *status, cudaStream_t st)
{
    using L = F32Layout<N, BG, TWO>;
    constexpr int NT = BG * (N / ZS);
    const size_t smem = (size_t)STAGES * L::kStageBytes;
    auto kern = conv_f32_kernel<N, BG, ZS, STAGES, TWO>;
    cudaError_t e = cudaFuncSetAttribute(
        kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int groups = (B + BG - 1) / BG;
    dim3 grid(N * N, groups);
    kern<<<grid, NT, smem, st>>>(Wblk, P, R, S, T, qacc, flush, status);
    return cudaGetLastError();
}

template <int N, int BG, int STAGES, bool TWO>
cudaError_t dispatch_zs(const float *Wblk, const float2 *P, const float2 *R,
                        const float2 *S, const float2 *T, double2 *qacc, int B,
                        int flush, unsigned int *status, cudaStream_t st)
{
    // Registers: ZS accumulators plus a (ZS+7)-wide window per operand
    // row; TWO doubles the windows, so it takes the narrower split.
    constexpr int ZS = TWO ? 8 : (N >= 16 ? 16 : 8);
    constexpr int ZSe = (N % ZS == 0) ? ZS : 8;
    return launch_f32<N, BG, ZSe, STAGES, TWO>(Wblk, P, R, S, T, qacc, B, flush,
                                              status, st);
}

template <int N, bool TWO>
cudaError_t dispatch_bg(const float *Wblk, const float2 *P, const float2 *R,
                        const float2 *S, const float2 *T, double2 *qacc, int B,
                        ConvF32Config cfg, unsigned int *status,
                        cudaStream_t st)
{
#define SBTE_CASE(BGV, STV)                                                      \
    if (cfg.bg == BGV && cfg.stages == STV)                                      \
        return dispatch_zs<N, BGV, STV, TWO>(Wblk, P, R, S, T, qacc, B, cfg.flush, \
                                             status, st);
    SBTE_CASE(32, 2)
    SBTE_CASE(32, 3)
    SBTE_CASE(64, 2)
    SBTE_CASE(64, 3)
    SBTE_CASE(128, 2)
#undef SBTE_CASE
    return cudaErrorInvalidValue;
}

__global__ void tile_weights_kernel(const double *__restrict__ W,
                                    float *__restrict__ Wblk, int N)
{
    // Wblk[zrow][xrow][zz][xz] = (float) W[zrow*N + zz][xrow*N + xz]
    const long long nn = (long long)N * N;
    const long long n3 = nn * N;
    const long long total = n3 * n3;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long row = t / n3, col = t % n3;
        const long long zrow = row / N, zz = row % N;
        const long long xrow = col / N, xz = col % N;
        Wblk[((zrow * nn + xrow) * N + zz) * N + xz] = (float)W[t];
    }
}

// One CTA per zeta-row (zx, zy): list the run rows in order (sym_slots of
// them), then fill Wsym[zrow][slot][zz][xz].  FP64 sum, one FP32 rounding.
__global__ void sym_weights_kernel(const double *__restrict__ W, float *__restrict__ Wsym, int N)
{
    __shared__ short rows[64 * 64 / 2 + 2];
    __shared__ int nrows;
    const int nn = N * N, h = N / 2;
    const long long n3 = (long long)nn * N;
    const int zrow = blockIdx.x, zx = zrow / N, zy = zrow % N;
    const int ms = sym_max_slots(N);
    if (threadIdx.x == 0) {
        int k = 0;
        for (int r = 0; r < nn && k < ms; r++) {
            const int sx = (zx + h - r / N + N) % N, sy = (zy + h - r % N + N) % N;
            if (sx * N + sy >= r) rows[k++] = (short)r;
        }
        nrows = k;
    }
    __syncthreads();
    const int nr = nrows;
    float *out = Wsym + (long long)zrow * ms * nn;
    for (int t = threadIdx.x; t < ms * nn; t += blockDim.x) {
        const int slot = t / nn, zz = (t % nn) / N, xz = t % N;
        double w = 0.0;
        if (slot < nr) {
            const int r = rows[slot];
            const int sx = (zx + h - r / N + N) % N, sy = (zy + h - r % N + N) % N;
            const int sr = sx * N + sy;
            const long long zrow_off = ((long long)zrow * N + zz) * n3;
            w = W[zrow_off + (long long)r * N + xz];
            if (sr != r) {
                const int sz = (zz + h - xz + N) % N;
                w += W[zrow_off + (long long)sr * N + sz];
            }
        }
        out[t] = (float)w;
    }
}

__global__ void tile_weights_x2_kernel(const double *__restrict__ W,
                                       float2 *__restrict__ W2, int N)
{
    // W2[zrow][xrow][zz][xz] = ((float) w, (float) w)
    const long long nn = (long long)N * N;
    const long long n3 = nn * N;
    const long long total = n3 * n3;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long row = t / n3, col = t % n3;
        const long long zrow = row / N, zz = row % N;
        const long long xrow = col / N, xz = col % N;
        const float w = (float)W[t];
        W2[((zrow * nn + xrow) * N + zz) * N + xz] = make_float2(w, w);
    }
}

}  // namespace

cudaError_t weights_to_tiled_f32x2(const double *W, float2 *W2blk, int N, cudaStream_t st)
{
    tile_weights_x2_kernel<<<152 * 8, 256, 0, st>>>(W, W2blk, N);
    return cudaGetLastError();
}

cudaError_t conv_f64(const double *W, const double2 *P, const double2 *R,
                     const double2 *S, const double2 *T, double2 *qhat, int N,
                     int B, cudaStream_t st)
{
    if (N < 2 || B < 1 || B > 65535) return cudaErrorInvalidValue;
    const long long n3 = (long long)N * N * N;
    const int wpb = 8;
    dim3 grid((unsigned)((n3 + wpb - 1) / wpb), B);
    if (S)
        conv_f64_kernel<true><<<grid, wpb * 32, 0, st>>>(W, P, R, S, T, qhat, N);
    else
        conv_f64_kernel<false><<<grid, wpb * 32, 0, st>>>(W, P, R, S, T, qhat, N);
    return cudaGetLastError();
}

// CTAs per SM the register budget of a warp-specialised shape is sized for:
// variant 5 caps it for two CTAs of 64 instances or three of 32.
static int ws_minb(const ConvF32Config &cfg)
{
    return cfg.variant == 5 ? (cfg.bg == 32 ? 3 : 2) : 1;
}

bool conv_f32_supported(int N, ConvF32Config cfg, bool two_pairs)
{
    if (cfg.variant == 2 || cfg.variant == 3 || cfg.variant == 5)
        return conv_ws_supported(N, cfg.bg, cfg.zs, cfg.variant == 2, cfg.stages, two_pairs,
                                 ws_minb(cfg));
    if (cfg.variant == 4) return conv_x4_supported(N, cfg.bg, cfg.zs, cfg.stages, two_pairs);
    if (cfg.variant != 1) return false;
    if (!(N == 8 || N == 16 || N == 24 || N == 32)) return false;
    const bool ok = (cfg.bg == 32 && (cfg.stages == 2 || cfg.stages == 3)) ||
                    (cfg.bg == 64 && (cfg.stages == 2 || cfg.stages == 3)) ||
                    (cfg.bg == 128 && cfg.stages == 2);
    return ok && conv_f32_smem_bytes(N, cfg, two_pairs) <= 227 * 1024;
}

size_t conv_f32_smem_bytes(int N, ConvF32Config cfg, bool two_pairs)
{
    const size_t rows = two_pairs ? 4 : 2;
    return (size_t)cfg.stages * ((size_t)N * N * 4 + rows * (size_t)N * cfg.bg * 8);
}

cudaError_t conv_f32_batched(const float *Wblk, const float2 *P,
                             const float2 *R, const float2 *S,
                             const float2 *T, double2 *qacc, int N, int B,
                             ConvF32Config cfg, unsigned int *status,
                             cudaStream_t st)
{
    const bool two = (S != nullptr);
    if (!conv_f32_supported(N, cfg, two) || B < 1) return cudaErrorInvalidValue;
    if (cfg.variant == 2 || cfg.variant == 3 || cfg.variant == 5)
        return conv_ws(Wblk, P, R, S, T, qacc, N, B, cfg.bg, cfg.zs, cfg.variant == 2,
                       cfg.stages, cfg.flush, cfg.sym, ws_minb(cfg), status, st,
                       cfg.stall_slot, cfg.stall_limit);
    if (cfg.sym) return cudaErrorInvalidValue;  // the symmetric form is variants 2, 3, 5 only
    switch (N) {
    case 8:
        return two ? dispatch_bg<8, true>(Wblk, P, R, S, T, qacc, B, cfg, status, st)
                   : dispatch_bg<8, false>(Wblk, P, R, S, T, qacc, B, cfg, status, st);
    case 16:
        return two ? dispatch_bg<16, true>(Wblk, P, R, S, T, qacc, B, cfg, status, st)
                   : dispatch_bg<16, false>(Wblk, P, R, S, T, qacc, B, cfg, status, st);
    case 24:
        return two ? dispatch_bg<24, true>(Wblk, P, R, S, T, qacc, B, cfg, status, st)
                   : dispatch_bg<24, false>(Wblk, P, R, S, T, qacc, B, cfg, status, st);
    case 32:
        return two ? dispatch_bg<32, true>(Wblk, P, R, S, T, qacc, B, cfg, status, st)
                   : dispatch_bg<32, false>(Wblk, P, R, S, T, qacc, B, cfg, status, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t weights_to_tiled_f32(const double *W, float *Wblk, int N,
                                 cudaStream_t st)
{
    tile_weights_kernel<<<152 * 8, 256, 0, st>>>(W, Wblk, N);
    return cudaGetLastError();
}

cudaError_t weights_to_sym_f32(const double *W, float *Wsym, int N, cudaStream_t st)
{
    if (N % 2 != 0 || N > 64 || N < 2) return cudaErrorInvalidValue;
    sym_weights_kernel<<<N * N, 256, 0, st>>>(W, Wsym, N);
    return cudaGetLastError();
}

}  // namespace sbte
