// conv_ws.cu -- the batched FP32 convolution of compute_Qhat
// (collisions.c:125-165), warp-specialised, with packed FP32x2 arithmetic.
//
// Work split: the same as conv_f32_kernel.  A CTA owns one zeta-row
// (zx, zy; all zz) for a group of bg instances in the bg-interleaved layout,
// and steps through the N^2 xi-rows.  What differs:
//  * Producer/consumer pipeline.  One producer warp fills a stages-deep ring
//    with 1-D bulk copies (cp.async.bulk).  Each stage holds the W tile, the
//    ghat row and the fhat row of the whole instance group.  Per stage, a
//    "full" mbarrier counts the bytes in and an "empty" mbarrier collects
//    one arrival per consumer warp.  Consumer warps wait only on data, and
//    the block never runs a __syncthreads inside the loop.
//  * Packed FP32x2 math.  One term W * g * f, with complex g and f and real
//    W, costs three f32x2 instructions:
//      t   = (g.x, g.x) * (f.x, f.y)
//      t  += (-g.y, g.y) * (f.y, f.x)
//      acc += (w, w) * t
//    That is half the issue slots of the six scalar instructions, with the
//    same FMA-pipe work, so the pipe rather than instruction issue sets the
//    speed.
//  * Wrap-free window.  The fhat row lands in shared memory together with
//    the first entries of a second copy, so each thread's sliding window
//    fhat[(zeta_z + N/2 - xi_z) mod N] is one contiguous run.  No per-element
//    wrap arithmetic remains.
//  * FP32 partial sums go to an FP64 accumulator every `flush` xi-rows.  The
//    first flush stores, later flushes add, so no memset is needed.
//  * Symmetric form (sym != 0).  For a fixed zeta the partner map
//    sigma(xi) = (zeta + N/2 - xi) mod N (per axis) is an involution, and the
//    product the sum weights is symmetric in (xi, sigma(xi)) whenever g = f:
//    ghat[xi] fhat[sigma xi] for Q(f,f), and ghat[xi] fhat[sigma xi] +
//    Mhat[xi] ghat[sigma xi] with fhat = Mhat + ghat for the maxPreserve sum.
//    So the xi-rows pair up as (r, sigma(r)), and one pass over row r with
//    the tile W[zeta][r][zz][xz] + W[zeta][sigma r][zz][sigma_z(xz)] covers
//    both.  The producer skips every row whose partner precedes it, and the
//    CTA runs (N^2 + F)/2 slots instead of N^2, where F (0 or 4) counts the
//    rows that are their own partner.  Wblk is then the pre-summed table of
//    weights_to_sym_f32.
//  * Bounded waits.  Every mbarrier wait gives up after a clock limit, sets
//    kStatusTimeout in the status word and leaves; before leaving, the
//    producer and the consumers wait (again bounded) for the copies already
//    issued into the ring, so no copy lands in the shared memory of a CTA
//    that has exited.  A test hook (stall_slot >= 0) makes the producer of
//    CTA (0, 0) skip that slot's copies, and that CTA's waits use stall_limit
//    clocks: its consumers then wait on a barrier that nothing completes,
//    which is how the timeout path is tested without a fault.
#include "common.cuh"
#include "kernels.h"
#include "mbarrier.cuh"

#include <cstdint>

namespace sbte {
namespace {

// PACKED: FP32x2 math with the fhat row stored with its wrapped head
// (window needs no wrap arithmetic); otherwise scalar FP32 math on a plain
// row with the wrap folded into the window index.
template <int N, int BG, int ZS, bool TWO, bool PACKED, int ST>
struct WsLayout {
    static constexpr int kNeed = PACKED ? N + ZS + 6 : N;  // window entries
    static constexpr int kWBytes = N * N * 4;
    static constexpr int kRowBytes = N * BG * 8;      // one row, all instances
    static constexpr int kWinBytes = kNeed * BG * 8;  // row (+ wrapped head)
    static constexpr int kStageBytes =
        kWBytes + kRowBytes + kWinBytes + (TWO ? kRowBytes + kWinBytes : 0);
    static constexpr int kStages = ST;
    static constexpr int kConsumers = BG * (N / ZS);
    static constexpr int kThreads = kConsumers + 32;
};

__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

template <int N, int BG, int ZS, bool TWO, bool PACKED, int STG, int MINB>
__global__ void __launch_bounds__(WsLayout<N, BG, ZS, TWO, PACKED, STG>::kThreads, MINB)
conv_ws_kernel(const float *__restrict__ Wblk, const float2 *__restrict__ P,
               const float2 *__restrict__ R, const float2 *__restrict__ S,
               const float2 *__restrict__ T, double2 *__restrict__ qacc, int flush, int sym,
               unsigned int *__restrict__ status, int stall_slot, long long stall_limit)
{
    using L = WsLayout<N, BG, ZS, TWO, PACKED, STG>;
    constexpr int NN = N * N;
    constexpr int H = N / 2;
    constexpr int ST = L::kStages;
    constexpr int NCW = L::kConsumers / 32;
    constexpr long long N3 = (long long)NN * N;
    static_assert(N % 8 == 0 && N % ZS == 0 && BG % 32 == 0, "shape");
    static_assert(L::kNeed <= 3 * N, "window fits in three row copies");

    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[ST];
    __shared__ uint64_t empty[ST];

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int zrow = blockIdx.x;
    const int zx = zrow / N, zy = zrow % N;
    const long long grp = blockIdx.y;
    // slots this CTA runs: every xi-row, or one per partner pair
    const int nslot = sym ? sym_slots(N, zx, zy) : NN;
    // the stall test hook acts on CTA (0, 0) only; every other CTA keeps the
    // default limit and skips nothing
    const bool stall_cta = stall_slot >= 0 && blockIdx.x == 0 && blockIdx.y == 0;
    const int skip = stall_cta ? stall_slot : -1;
    const long long limit = stall_cta ? stall_limit : kWaitLimitClocks;

    if (tid == 0) {
        for (int s = 0; s < ST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NCW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        // ------------------------------------------------------ producer
        if ((tid & 31) != 0) return;
        const float *Wbase = Wblk + (long long)zrow * (sym ? sym_max_slots(N) : NN) * NN;
        const float2 *Pg = P + grp * N3 * BG;
        const float2 *Rg = R + grp * N3 * BG;
        const float2 *Sg = TWO ? S + grp * N3 * BG : nullptr;
        const float2 *Tg = TWO ? T + grp * N3 * BG : nullptr;
        int slot = 0;
        for (int it = 0; it < NN && slot < nslot; it++) {
            const int xx = it / N, xy = it % N;
            const int fx = (zx + H - xx < 0) ? zx + H - xx + N
                           : (zx + H - xx > N - 1 ? zx + H - xx - N : zx + H - xx);
            const int fy = (zy + H - xy < 0) ? zy + H - xy + N
                           : (zy + H - xy > N - 1 ? zy + H - xy - N : zy + H - xy);
            if (sym && fx * N + fy < it) continue;  // covered by its partner row
            const int s = slot % ST;
            if (slot >= ST) {
                if (!mbar_wait_bounded(&empty[s], (uint32_t)(((slot / ST) - 1) & 1), limit)) {
                    atomicOr(status, kStatusTimeout);
                    // let the copies of the slots issued since land before
                    // this thread, and with it the CTA, leaves
                    for (int j = slot - ST + 1; j < slot; j++)
                        if (j != skip)
                            (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1),
                                                    limit);
                    return;
                }
            }
            if (slot == skip) {  // test hook: this slot's barrier never completes
                slot++;
                continue;
            }
            unsigned char *base = smem + s * L::kStageBytes;
            const long long prow = (long long)it * N * BG;
            const long long rrow = ((long long)fx * N + fy) * N * BG;
            mbar_expect_tx(&full[s], L::kStageBytes);
            unsigned char *d = base;
            bulk_g2s(d, Wbase + (long long)slot * NN, L::kWBytes, &full[s]);
            slot++;
            d += L::kWBytes;
            bulk_g2s(d, Pg + prow, L::kRowBytes, &full[s]);
            d += L::kRowBytes;
            // the fhat row, then its first kNeed - N entries again
            for (int done = 0; done < L::kNeed; done += N) {
                const int cnt = (L::kNeed - done < N) ? L::kNeed - done : N;
                bulk_g2s(d + (size_t)done * BG * 8, Rg + rrow, cnt * BG * 8, &full[s]);
            }
            d += L::kWinBytes;
            if (TWO) {
                bulk_g2s(d, Sg + prow, L::kRowBytes, &full[s]);
                d += L::kRowBytes;
                for (int done = 0; done < L::kNeed; done += N) {
                    const int cnt = (L::kNeed - done < N) ? L::kNeed - done : N;
                    bulk_g2s(d + (size_t)done * BG * 8, Tg + rrow, cnt * BG * 8, &full[s]);
                }
            }
        }
        return;
    }

    // ---------------------------------------------------------- consumers
    const int b = tid % BG;
    const int zq = tid / BG;
    const int z0 = zq * ZS;
    float2 acc[ZS];
#pragma unroll
    for (int i = 0; i < ZS; i++) acc[i] = f2(0.f, 0.f);
    double2 *qrow = qacc + grp * N3 * BG + ((long long)zrow * N + z0) * BG + b;
    bool first_flush = true;
    int since = 0;

    // The first flush stores; later ones add with fire-and-forget reductions
    // (red.global.add.f64), so the consumer never waits on a global load.
    // Each accumulator has a single writer, which adds in program order, so
    // the sum is deterministic.
    auto do_flush = [&]() {
#pragma unroll
        for (int i = 0; i < ZS; i++) {
            double2 *q = qrow + (long long)i * BG;
            if (first_flush) {
                *q = make_double2((double)acc[i].x, (double)acc[i].y);
            } else {
                atomicAdd(&q->x, (double)acc[i].x);
                atomicAdd(&q->y, (double)acc[i].y);
            }
            acc[i] = f2(0.f, 0.f);
        }
        first_flush = false;
    };

    for (int it = 0; it < nslot; it++) {
        const int s = it % ST;
        if (!mbar_wait_bounded(&full[s], (uint32_t)((it / ST) & 1), limit)) {
            atomicOr(status, kStatusTimeout);
            // The producer may have issued slots it + 1 .. it + ST - 1 (their
            // stages were released); give each copy a bounded chance to land
            // before leaving.  Slot `it` itself gets one more wait.
            for (int j = it; j < it + ST && j < nslot; j++)
                if (j != skip)
                    (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), limit);
            return;
        }
        const unsigned char *base = smem + s * L::kStageBytes;
        const float *Ws = reinterpret_cast<const float *>(base);
        const float2 *Gs = reinterpret_cast<const float2 *>(base + L::kWBytes);
        const float2 *Fs = reinterpret_cast<const float2 *>(base + L::kWBytes + L::kRowBytes);
        const float2 *Ss = reinterpret_cast<const float2 *>(base + L::kWBytes + L::kRowBytes +
                                                            L::kWinBytes);
        const float2 *Ts = reinterpret_cast<const float2 *>(base + L::kWBytes + 2 * L::kRowBytes +
                                                            L::kWinBytes);
#pragma unroll
        for (int c = 0; c < N / 8; c++) {
            float2 gxx[8], gyn[8];
            float2 sxx[TWO ? 8 : 1], syn[TWO ? 8 : 1];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                const float2 g = Gs[(8 * c + e) * BG + b];
                gxx[e] = f2(g.x, g.x);
                gyn[e] = f2(-g.y, g.y);
                if (TWO) {
                    const float2 q = Ss[(8 * c + e) * BG + b];
                    sxx[e] = f2(q.x, q.x);
                    syn[e] = f2(-q.y, q.y);
                }
            }
            // window start: (z0 + H - 8c - 7) mod N
            int start = z0 + H - 8 * c - 7;
            start = start < 0 ? start + N : (start >= N ? start - N : start);
            if constexpr (PACKED) {
                // contiguous: the row is followed by its wrapped head
                const float2 *Fw = Fs + start * BG + b;
                const float2 *Tw = Ts + start * BG + b;
                float2 fw[ZS + 7], fsw[ZS + 7];
                float2 tw[TWO ? ZS + 7 : 1], tsw[TWO ? ZS + 7 : 1];
#pragma unroll
                for (int d = 0; d < ZS + 7; d++) {
                    fw[d] = Fw[d * BG];
                    fsw[d] = f2(fw[d].y, fw[d].x);
                    if (TWO) {
                        tw[d] = Tw[d * BG];
                        tsw[d] = f2(tw[d].y, tw[d].x);
                    }
                }
#pragma unroll
                for (int zl = 0; zl < ZS; zl++) {
                    const float4 wa = *reinterpret_cast<const float4 *>(Ws + (z0 + zl) * N + 8 * c);
                    const float4 wb =
                        *reinterpret_cast<const float4 *>(Ws + (z0 + zl) * N + 8 * c + 4);
                    const float w[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        // zeta_z = z0+zl, xi_z = 8c+e  ->  window slot zl - e + 7
                        float2 t = __fmul2_rn(gxx[e], fw[zl - e + 7]);
                        t = __ffma2_rn(gyn[e], fsw[zl - e + 7], t);
                        if (TWO) {
                            t = __ffma2_rn(sxx[e], tw[zl - e + 7], t);
                            t = __ffma2_rn(syn[e], tsw[zl - e + 7], t);
                        }
                        acc[zl] = __ffma2_rn(f2(w[e], w[e]), t, acc[zl]);
                    }
                }
            } else {
                float2 fw[ZS + 7];
                float2 tw[TWO ? ZS + 7 : 1];
                int zi = start;
#pragma unroll
                for (int d = 0; d < ZS + 7; d++) {
                    fw[d] = Fs[zi * BG + b];
                    if (TWO) tw[d] = Ts[zi * BG + b];
                    zi = (zi == N - 1) ? 0 : zi + 1;
                }
#pragma unroll
                for (int zl = 0; zl < ZS; zl++) {
                    const float4 wa = *reinterpret_cast<const float4 *>(Ws + (z0 + zl) * N + 8 * c);
                    const float4 wb =
                        *reinterpret_cast<const float4 *>(Ws + (z0 + zl) * N + 8 * c + 4);
                    const float w[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
                    for (int e = 0; e < 8; e++) {
                        const float2 f = fw[zl - e + 7];
                        const float gx = gxx[e].x, gy = gyn[e].y;
                        float pr = gx * f.x;
                        pr = fmaf(-gy, f.y, pr);
                        float pi = gx * f.y;
                        pi = fmaf(gy, f.x, pi);
                        if (TWO) {
                            const float2 t = tw[zl - e + 7];
                            const float sx = sxx[e].x, sy = syn[e].y;
                            pr = fmaf(sx, t.x, pr);
                            pr = fmaf(-sy, t.y, pr);
                            pi = fmaf(sx, t.y, pi);
                            pi = fmaf(sy, t.x, pi);
                        }
                        acc[zl].x = fmaf(w[e], pr, acc[zl].x);
                        acc[zl].y = fmaf(w[e], pi, acc[zl].y);
                    }
                }
            }
        }
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&empty[s]);
        if (++since == flush) {
            do_flush();
            since = 0;
        }
    }
    if (since || first_flush) do_flush();
}

template <int N, int BG, int ZS, bool TWO, bool PACKED, int ST, int MINB>
cudaError_t launch_ws(const float *Wblk, const float2 *P, const float2 *R, const float2 *S,
                      const float2 *T, double2 *qacc, int B, int flush, int sym, unsigned *status,
                      cudaStream_t st, int stall_slot, long long stall_limit)
{
    using L = WsLayout<N, BG, ZS, TWO, PACKED, ST>;
    const size_t smem = (size_t)L::kStages * L::kStageBytes;
    auto kern = conv_ws_kernel<N, BG, ZS, TWO, PACKED, ST, MINB>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(N * N, (B + BG - 1) / BG);
    kern<<<grid, L::kThreads, smem, st>>>(Wblk, P, R, S, T, qacc, flush, sym, status,
                                          stall_slot, stall_limit);
    return cudaGetLastError();
}

template <int N, int BG, int ZS, bool TWO, bool PACKED, int ST>
size_t ws_smem()
{
    using L = WsLayout<N, BG, ZS, TWO, PACKED, ST>;
    return (size_t)L::kStages * L::kStageBytes;
}

}  // namespace

// Shapes instantiated for the warp-specialised kernel:
// (N, bg, zs, packed, stages, minb); variant 2 = packed FP32x2, 3 = scalar,
// N = 48 for the row-pair table of the closed-form weights (no FP64 table);
// 5 = scalar with the registers capped so that minb = 2 CTAs fit on an SM
// (96 registers at N = 32, bg = 64, no spill; uncapped, variant 3 takes 146
// and one CTA per SM; a cap of 3 CTAs (72 registers) spilled and ran 3%
// slower), or minb = 3 at bg = 32 (128 registers, the same speed per
// instance), which serves calls of at most 32 instances.
#define SBTE_WS_SHAPES(X)                                                                 \
    X(8, 32, 8, 1, 2, 1) X(8, 32, 8, 0, 3, 1) X(8, 64, 8, 0, 3, 1)                        \
    X(16, 32, 8, 1, 2, 1) X(16, 32, 8, 0, 3, 1) X(16, 64, 8, 0, 3, 1) X(16, 64, 16, 0, 3, 1) \
    X(24, 32, 8, 1, 2, 1) X(24, 32, 8, 0, 3, 1) X(24, 64, 8, 0, 2, 1) X(24, 64, 8, 0, 3, 1)  \
    X(32, 32, 8, 1, 2, 1) X(32, 64, 8, 1, 2, 1) X(32, 32, 8, 0, 3, 1) X(32, 64, 8, 0, 2, 1)  \
    X(32, 64, 8, 0, 3, 1) X(32, 64, 16, 0, 2, 1) X(32, 64, 16, 0, 3, 1)                   \
    X(32, 64, 8, 0, 2, 2) X(32, 64, 8, 0, 3, 2) X(32, 32, 8, 0, 2, 3) X(32, 32, 8, 0, 3, 3)     \
    X(48, 32, 8, 0, 3, 1) X(48, 64, 8, 0, 2, 1)

bool conv_ws_supported(int N, int bg, int zs, bool packed, int stages, bool two, int minb)
{
    // the two-pair form does not fit the capped register budget (it spills)
    if (two && minb != 1) return false;
#define SBTE_WS_Q(NN, BGV, ZSV, PK, STV, MB)                                             \
    if (N == NN && bg == BGV && zs == ZSV && packed == (PK != 0) && stages == STV &&    \
        minb == MB)                                                                      \
        return (two ? ws_smem<NN, BGV, ZSV, true, PK != 0, STV>()                       \
                    : ws_smem<NN, BGV, ZSV, false, PK != 0, STV>()) <= 227 * 1024;
    SBTE_WS_SHAPES(SBTE_WS_Q)
#undef SBTE_WS_Q
    return false;
}

cudaError_t conv_ws(const float *Wblk, const float2 *P, const float2 *R, const float2 *S,
                    const float2 *T, double2 *qacc, int N, int B, int bg, int zs, bool packed,
                    int stages, int flush, int sym, int minb, unsigned int *status,
                    cudaStream_t st, int stall_slot, long long stall_limit)
{
    const bool two = (S != nullptr);
    if (!conv_ws_supported(N, bg, zs, packed, stages, two, minb) || B < 1)
        return cudaErrorInvalidValue;
    if (stall_slot >= 0 && stall_limit <= 0) return cudaErrorInvalidValue;
#define SBTE_WS_L(NN, BGV, ZSV, PK, STV, MB)                                                  \
    if (N == NN && bg == BGV && zs == ZSV && packed == (PK != 0) && stages == STV &&         \
        minb == MB)                                                                           \
        return two ? launch_ws<NN, BGV, ZSV, true, PK != 0, STV, MB>(                       \
                         Wblk, P, R, S, T, qacc, B, flush, sym, status, st, stall_slot,         \
                         stall_limit)                                                           \
                   : launch_ws<NN, BGV, ZSV, false, PK != 0, STV, MB>(                      \
                         Wblk, P, R, S, T, qacc, B, flush, sym, status, st, stall_slot,         \
                         stall_limit);
    SBTE_WS_SHAPES(SBTE_WS_L)
#undef SBTE_WS_L
    return cudaErrorInvalidValue;
}

}  // namespace sbte

// ======================================================================
// Variant 4: packed FP32x2 math with expanded operands.  The FFT writes
// ghat as (g.x, g.x, -g.y, g.y) and fhat as (f.x, f.y, f.y, f.x), and W is
// tiled as (w, w) pairs.  Every 128-bit shared load then hands the math two
// ready-made 64-bit operand pairs, so one term costs three f32x2
// instructions and no register moves.
// ======================================================================
namespace sbte {
namespace {

template <int N, int BG, int ZS, bool TWO, int ST>
struct X4Layout {
    static constexpr int kNeed = N + ZS + 6;          // window entries incl. wrap
    static constexpr int kWBytes = N * N * 8;         // (w, w) pairs
    static constexpr int kRowBytes = N * BG * 16;     // one G4 row
    static constexpr int kWinBytes = kNeed * BG * 16; // F4 row + wrapped head
    static constexpr int kStageBytes =
        kWBytes + kRowBytes + kWinBytes + (TWO ? kRowBytes + kWinBytes : 0);
    static constexpr int kConsumers = BG * (N / ZS);
    static constexpr int kThreads = kConsumers + 32;
};

__device__ __forceinline__ float2 lo2(float4 q) { return make_float2(q.x, q.y); }
__device__ __forceinline__ float2 hi2(float4 q) { return make_float2(q.z, q.w); }

template <int N, int BG, int ZS, bool TWO, int ST>
__global__ void __launch_bounds__(X4Layout<N, BG, ZS, TWO, ST>::kThreads)
conv_x4_kernel(const float2 *__restrict__ W2blk, const float4 *__restrict__ P,
               const float4 *__restrict__ R, const float4 *__restrict__ S,
               const float4 *__restrict__ T, double2 *__restrict__ qacc, int flush,
               unsigned int *__restrict__ status)
{
    using L = X4Layout<N, BG, ZS, TWO, ST>;
    constexpr int NN = N * N;
    constexpr int H = N / 2;
    constexpr int NCW = L::kConsumers / 32;
    constexpr long long N3 = (long long)NN * N;
    static_assert(N % 8 == 0 && N % ZS == 0 && BG % 32 == 0, "shape");
    static_assert(L::kNeed <= 3 * N, "window fits in three row copies");

    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t full[ST];
    __shared__ uint64_t empty[ST];

    const int tid = threadIdx.x;
    const int warp = tid >> 5;
    const int zrow = blockIdx.x;
    const int zx = zrow / N, zy = zrow % N;
    const long long grp = blockIdx.y;

    if (tid == 0) {
        for (int s = 0; s < ST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], NCW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        if ((tid & 31) != 0) return;
        const float2 *Wbase = W2blk + (long long)zrow * NN * NN;
        const float4 *Pg = P + grp * N3 * BG;
        const float4 *Rg = R + grp * N3 * BG;
        const float4 *Sg = TWO ? S + grp * N3 * BG : nullptr;
        const float4 *Tg = TWO ? T + grp * N3 * BG : nullptr;
        for (int it = 0; it < NN; it++) {
            const int s = it % ST;
            if (it >= ST) {
                if (!mbar_wait_bounded(&empty[s], (uint32_t)(((it / ST) - 1) & 1))) {
                    atomicOr(status, kStatusTimeout);
                    return;
                }
            }
            unsigned char *d = smem + s * L::kStageBytes;
            const int xx = it / N, xy = it % N;
            const int fx = (zx + H - xx < 0) ? zx + H - xx + N
                           : (zx + H - xx > N - 1 ? zx + H - xx - N : zx + H - xx);
            const int fy = (zy + H - xy < 0) ? zy + H - xy + N
                           : (zy + H - xy > N - 1 ? zy + H - xy - N : zy + H - xy);
            const long long prow = (long long)it * N * BG;
            const long long rrow = ((long long)fx * N + fy) * N * BG;
            mbar_expect_tx(&full[s], L::kStageBytes);
            bulk_g2s(d, Wbase + (long long)it * NN, L::kWBytes, &full[s]);
            d += L::kWBytes;
            bulk_g2s(d, Pg + prow, L::kRowBytes, &full[s]);
            d += L::kRowBytes;
            for (int done = 0; done < L::kNeed; done += N) {
                const int cnt = (L::kNeed - done < N) ? L::kNeed - done : N;
                bulk_g2s(d + (size_t)done * BG * 16, Rg + rrow, cnt * BG * 16, &full[s]);
            }
            d += L::kWinBytes;
            if (TWO) {
                bulk_g2s(d, Sg + prow, L::kRowBytes, &full[s]);
                d += L::kRowBytes;
                for (int done = 0; done < L::kNeed; done += N) {
                    const int cnt = (L::kNeed - done < N) ? L::kNeed - done : N;
                    bulk_g2s(d + (size_t)done * BG * 16, Tg + rrow, cnt * BG * 16, &full[s]);
                }
            }
        }
        return;
    }

    const int b = tid % BG;
    const int zq = tid / BG;
    const int z0 = zq * ZS;
    float2 acc[ZS];
#pragma unroll
    for (int i = 0; i < ZS; i++) acc[i] = make_float2(0.f, 0.f);
    double2 *qrow = qacc + grp * N3 * BG + ((long long)zrow * N + z0) * BG + b;
    bool first_flush = true;
    int since = 0;
    auto do_flush = [&]() {
#pragma unroll
        for (int i = 0; i < ZS; i++) {
            double2 q = first_flush ? make_double2(0.0, 0.0) : qrow[(long long)i * BG];
            q.x += (double)acc[i].x;
            q.y += (double)acc[i].y;
            qrow[(long long)i * BG] = q;
            acc[i] = make_float2(0.f, 0.f);
        }
        first_flush = false;
    };

    for (int it = 0; it < NN; it++) {
        const int s = it % ST;
        if (!mbar_wait_bounded(&full[s], (uint32_t)((it / ST) & 1))) {
            atomicOr(status, kStatusTimeout);
            (void)mbar_wait_bounded(&full[s], (uint32_t)((it / ST) & 1));
            return;
        }
        const unsigned char *base = smem + s * L::kStageBytes;
        const float4 *W4 = reinterpret_cast<const float4 *>(base);
        const float4 *G4 = reinterpret_cast<const float4 *>(base + L::kWBytes);
        const float4 *F4 = reinterpret_cast<const float4 *>(base + L::kWBytes + L::kRowBytes);
        const float4 *S4 = reinterpret_cast<const float4 *>(base + L::kWBytes + L::kRowBytes +
                                                            L::kWinBytes);
        const float4 *T4 = reinterpret_cast<const float4 *>(base + L::kWBytes +
                                                            2 * L::kRowBytes + L::kWinBytes);
#pragma unroll
        for (int c = 0; c < N / 8; c++) {
            float4 gq[8];
            float4 sq[TWO ? 8 : 1];
#pragma unroll
            for (int e = 0; e < 8; e++) {
                gq[e] = G4[(8 * c + e) * BG + b];
                if (TWO) sq[e] = S4[(8 * c + e) * BG + b];
            }
            int start = z0 + H - 8 * c - 7;
            start = start < 0 ? start + N : (start >= N ? start - N : start);
            float4 fq[ZS + 7];
            float4 tq[TWO ? ZS + 7 : 1];
#pragma unroll
            for (int d = 0; d < ZS + 7; d++) {
                fq[d] = F4[(start + d) * BG + b];
                if (TWO) tq[d] = T4[(start + d) * BG + b];
            }
#pragma unroll
            for (int zl = 0; zl < ZS; zl++) {
                // 8 (w, w) pairs of row z0+zl, columns 8c..8c+7
                float4 wq[4];
#pragma unroll
                for (int m = 0; m < 4; m++) wq[m] = W4[((z0 + zl) * N + 8 * c) / 2 + m];
#pragma unroll
                for (int e = 0; e < 8; e++) {
                    const float4 f = fq[zl - e + 7];
                    float2 t = __fmul2_rn(lo2(gq[e]), lo2(f));
                    t = __ffma2_rn(hi2(gq[e]), hi2(f), t);
                    if (TWO) {
                        const float4 tt = tq[zl - e + 7];
                        t = __ffma2_rn(lo2(sq[e]), lo2(tt), t);
                        t = __ffma2_rn(hi2(sq[e]), hi2(tt), t);
                    }
                    const float2 ww = (e & 1) ? hi2(wq[e >> 1]) : lo2(wq[e >> 1]);
                    acc[zl] = __ffma2_rn(ww, t, acc[zl]);
                }
            }
        }
        __syncwarp();
        if ((tid & 31) == 0) mbar_arrive(&empty[s]);
        if (++since == flush) {
            do_flush();
            since = 0;
        }
    }
    if (since || first_flush) do_flush();
}

template <int N, int BG, int ZS, bool TWO, int ST>
cudaError_t launch_x4(const float2 *W2, const float4 *P, const float4 *R, const float4 *S,
                      const float4 *T, double2 *qacc, int B, int flush, unsigned *status,
                      cudaStream_t st)
{
    using L = X4Layout<N, BG, ZS, TWO, ST>;
    const size_t smem = (size_t)ST * L::kStageBytes;
    auto kern = conv_x4_kernel<N, BG, ZS, TWO, ST>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid(N * N, (B + BG - 1) / BG);
    kern<<<grid, L::kThreads, smem, st>>>(W2, P, R, S, T, qacc, flush, status);
    return cudaGetLastError();
}

template <int N, int BG, int ZS, bool TWO, int ST>
size_t x4_smem()
{
    return (size_t)ST * X4Layout<N, BG, ZS, TWO, ST>::kStageBytes;
}

}  // namespace

#define SBTE_X4_SHAPES(X)                                                     \
    X(8, 32, 8, 2) X(16, 32, 8, 2) X(24, 32, 8, 2) X(32, 32, 8, 2)             \
    X(32, 64, 8, 2) X(32, 32, 8, 3)

bool conv_x4_supported(int N, int bg, int zs, int stages, bool two)
{
#define SBTE_X4_Q(NN, BGV, ZSV, STV)                                                  \
    if (N == NN && bg == BGV && zs == ZSV && stages == STV)                           \
        return (two ? x4_smem<NN, BGV, ZSV, true, STV>()                              \
                    : x4_smem<NN, BGV, ZSV, false, STV>()) <= 227 * 1024;
    SBTE_X4_SHAPES(SBTE_X4_Q)
#undef SBTE_X4_Q
    return false;
}

cudaError_t conv_x4(const float2 *W2blk, const float4 *P, const float4 *R, const float4 *S,
                    const float4 *T, double2 *qacc, int N, int B, int bg, int zs, int stages,
                    int flush, unsigned int *status, cudaStream_t st)
{
    const bool two = (S != nullptr);
    if (!conv_x4_supported(N, bg, zs, stages, two) || B < 1) return cudaErrorInvalidValue;
#define SBTE_X4_L(NN, BGV, ZSV, STV)                                                      \
    if (N == NN && bg == BGV && zs == ZSV && stages == STV)                               \
        return two ? launch_x4<NN, BGV, ZSV, true, STV>(W2blk, P, R, S, T, qacc, B, flush,  \
                                                        status, st)                        \
                   : launch_x4<NN, BGV, ZSV, false, STV>(W2blk, P, R, S, T, qacc, B, flush, \
                                                         status, st);
    SBTE_X4_SHAPES(SBTE_X4_L)
#undef SBTE_X4_L
    return cudaErrorInvalidValue;
}

}  // namespace sbte
