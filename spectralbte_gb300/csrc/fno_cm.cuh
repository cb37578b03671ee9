// fno_cm.cuh -- the channel mix of a spectral layer for inference,
// warp-specialised around the tensor memory accelerator (TMA):
//
//   h'[p][d][b] = act(sum_c W[d][c] h[p][c][b] + bias[d] + S[p][d][b])
//
// for 64 channels, activations [point][channel][instance] in 16-bit
// elements, Bp (instances, padded) a multiple of 64.  One work item is one
// point p and 64 instances: a 64 x 64 input tile of h and the same tile of
// the spectral sum S, 16 KB in all, and a 64 x 64 output tile.
//
//  * One producer warp (one elected thread) loads both tiles of an item with
//    two 2D TMA copies (cp.async.bulk.tensor, 128-byte swizzle) into a
//    ST-deep ring, each stage guarded by a "full" mbarrier (transaction
//    bytes) and an "empty" mbarrier (one arrival per consumer warp).
//  * 4 RW consumer warps: warp (wr, wc) owns output rows [64/RW wr, +64/RW)
//    and instance columns [16 wc, +16): its 64/RW x 16 block of the product on
//    the tensor cores (mma.sync m16n8k16, FP32 accumulation, W resident in
//    shared memory), then bias + S + GELU in registers, the 16-bit result
//    into a per-warp staging tile, and a 2D TMA store of that tile
//    (cp.async.bulk.tensor ... bulk_group), double buffered so the store
//    overlaps the next item.
//  * No block-wide barrier inside the loop: warps only wait on mbarriers, and
//    every wait is bounded.  A wait that runs out sets kStatusTimeout in the
//    status word and the thread drains its own outstanding copies before it
//    leaves.
// The swizzle: with 128-byte rows, TMA stores the 16-byte chunk c of row r at
// chunk c ^ (r & 7) (stage tiles are 1024-byte aligned), so the transposed
// ldmatrix of 8 rows and the epilogue's reads of S hit 8 distinct chunks.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>

#include "common.cuh"
#include "fno_gemm.cuh"
#include "mbarrier.cuh"

namespace sbte {
namespace fno {

constexpr int kCmC = 64;        // channels in and out
constexpr int kCmBN = 64;       // instances per item

template <int ST, int RW, int SB = 2> struct CmLayout {
    static constexpr int kWarps = 4 * RW;                     // consumer warps
    static constexpr int kThreads = 32 * (kWarps + 1);
    static constexpr int kRows = kCmC / RW;                   // output rows per warp
    static constexpr int kTile = kCmC * kCmBN * 2;            // 8 KB, one 16-bit tile
    static constexpr int kStage = 2 * kTile;                  // h tile + S tile
    static constexpr int kWP = kCmC + 8;                      // padded W row (elements)
    static constexpr int kW = kCmC * kWP * 2;                 // 9 KB
    static constexpr int kStg = kRows * 16 * 2;               // rows x 16 columns, 16-bit
    static constexpr size_t kStageOff = 0;
    static constexpr size_t kWOff = (size_t)ST * kStage;
    static constexpr size_t kStgOff = kWOff + kW;
    static constexpr size_t kBytes = kStgOff + (size_t)kWarps * SB * kStg;
    static constexpr size_t kAlloc = kBytes + 1024;           // room to align the base
};

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int x,
                                             int y)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;"); }
__device__ __forceinline__ void bulk_wait_read1()
{
    asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read0()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <typename E, int ST, int RW, int MINB, int SB = 2>
__global__ void __launch_bounds__(CmLayout<ST, RW, SB>::kThreads, MINB)
cm_ws_kernel(const __grid_constant__ CUtensorMap tH, const __grid_constant__ CUtensorMap tS,
             const __grid_constant__ CUtensorMap tO, const float *__restrict__ W,
             const float *__restrict__ bias, int act, int nb, long long total,
             long long wait_limit, unsigned int *__restrict__ status)
{
    using T2 = typename Elem<E>::T2;
    using L = CmLayout<ST, RW, SB>;
    constexpr int kCmWarps = L::kWarps, kCmThreads = L::kThreads, FM = L::kRows / 16;
    extern __shared__ unsigned char cm_smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(cm_smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[ST], empty[ST];
    E *sW = reinterpret_cast<E *>(smem + L::kWOff);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < ST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], kCmWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // W (FP32 parameters) -> 16-bit, padded rows
    for (int e = tid; e < kCmC * kCmC; e += kCmThreads) {
        const int m = e / kCmC, k = e % kCmC;
        sW[m * L::kWP + k] = Elem<E>::cvt(W[e]);
    }
    __syncthreads();

    if (warp == kCmWarps) {
        // ------------------------------------------------------ producer
        if (lane != 0) return;
        long long it = 0;
        for (long long i = blockIdx.x; i < total; i += gridDim.x, it++) {
            const int s = (int)(it % ST);
            if (it >= ST &&
                !mbar_wait_bounded(&empty[s], (uint32_t)(((it / ST) - 1) & 1), wait_limit)) {
                atomicOr(status, kStatusTimeout);
                // drain: the stages issued since the one that never came back
                for (long long j = it - ST + 1; j < it; j++)
                    (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), wait_limit);
                return;
            }
            const int p = (int)(i / nb), b0 = (int)(i % nb) * kCmBN;
            unsigned char *st = smem + L::kStageOff + (size_t)s * L::kStage;
            mbar_expect_tx(&full[s], (uint32_t)L::kStage);
            tma_load_2d(st, &tH, b0, p * kCmC, &full[s]);
            tma_load_2d(st + L::kTile, &tS, b0, p * kCmC, &full[s]);
        }
        return;
    }

    // ---------------------------------------------------------- consumers
    const int g = lane >> 2, t = lane & 3;
    const int col0 = (warp & 3) * 16;        // this warp's 16 columns of the 64
    const int row0 = (warp >> 2) * L::kRows;  // and its rows
    float bm[FM][2];
#pragma unroll
    for (int fm = 0; fm < FM; fm++) {
        bm[fm][0] = bias[row0 + 16 * fm + g];
        bm[fm][1] = bias[row0 + 16 * fm + g + 8];
    }
    E *stg0 = reinterpret_cast<E *>(smem + L::kStgOff + (size_t)warp * SB * L::kStg);
    long long it = 0;
    for (long long i = blockIdx.x; i < total; i += gridDim.x, it++) {
        const int s = (int)(it % ST);
        if (!mbar_wait_bounded(&full[s], (uint32_t)((it / ST) & 1), wait_limit)) {
            atomicOr(status, kStatusTimeout);
            for (long long j = it + 1; j < it + ST && j < total; j++)
                (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), wait_limit);
            if (lane == 0) bulk_wait_all();
            return;
        }
        const unsigned char *st = smem + L::kStageOff + (size_t)s * L::kStage;
        const E *sB = reinterpret_cast<const E *>(st);
        const unsigned char *sS = st + L::kTile;
        float acc[FM][2][4];
#pragma unroll
        for (int fm = 0; fm < FM; fm++)
#pragma unroll
            for (int fn = 0; fn < 2; fn++)
#pragma unroll
                for (int r = 0; r < 4; r++) acc[fm][fn][r] = 0.f;
#pragma unroll
        for (int kk = 0; kk < kCmC; kk += 16) {
            uint32_t a[FM][4], b[4];
#pragma unroll
            for (int fm = 0; fm < FM; fm++)
                ldsm_x4(a[fm], sW + (row0 + 16 * fm + (lane & 15)) * L::kWP + kk + (lane >> 4) * 8);
            const int krow = kk + (lane & 15);
            const int chunk = (col0 >> 3) + (lane >> 4);
            ldsm_x4_t(b, reinterpret_cast<const unsigned char *>(sB) + krow * 128 +
                             ((chunk ^ (krow & 7)) << 4));
#pragma unroll
            for (int fm = 0; fm < FM; fm++) {
                mma16816<E>(acc[fm][0], a[fm], b[0], b[1]);
                mma16816<E>(acc[fm][1], a[fm], b[2], b[3]);
            }
        }
        // the staging tile of this item: the store that last used it has read it
        E *stg = stg0 + (SB == 2 ? (it & 1) : 0) * (L::kRows * 16);
        if (lane == 0) {
            if (SB == 2)
                bulk_wait_read1();
            else
                bulk_wait_read0();
        }
        __syncwarp();
#pragma unroll
        for (int fm = 0; fm < FM; fm++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int ml = 16 * fm + g + 8 * hh;  // row in this warp's block
                const int m = row0 + ml;
#pragma unroll
                for (int fn = 0; fn < 2; fn++) {
                    const int c = col0 + 8 * fn + 2 * t;  // column in the 64-wide tile
                    const T2 sv = *reinterpret_cast<const T2 *>(
                        sS + m * 128 + ((((c >> 3) ^ (m & 7))) << 4) + (c & 7) * 2);
                    // (acc + bias) + S, then GELU: the general GEMM's
                    // epilogue in FP32x2 instructions, lane for lane
                    const float2 z = __fadd2_rn(
                        __fadd2_rn(make_float2(acc[fm][fn][2 * hh], acc[fm][fn][2 * hh + 1]),
                                   make_float2(bm[fm][hh], bm[fm][hh])),
                        Elem<E>::f2(sv));
                    const float2 o = act ? gelu2_f(z) : z;
                    *reinterpret_cast<T2 *>(stg + ml * 16 + 8 * fn + 2 * t) =
                        Elem<E>::cvt2(o.x, o.y);
                }
            }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
            mbar_arrive(&empty[s]);  // stage s read by this warp
            const int p = (int)(i / nb), b0 = (int)(i % nb) * kCmBN;
            tma_store_2d(&tO, stg, b0 + col0, p * kCmC + row0);
            bulk_commit();
        }
    }
    if (lane == 0) bulk_wait_all();
}

// ---------------------------------------------------------------------------
// The readout for inference, the same warp-specialised structure:
//   y[p][b] = c2 + sum_m q2[m] gelu(sum_c Q1[m][c] h[p][c][b] + c1[m])
// with 128 hidden rows m and 64 channels c.  A work item is one point and 64
// instances: one 64 x 64 tile of h (TMA, 128-byte swizzle) into the ring.
// Eight consumer warps: warp (wr, wc) computes hidden rows [64 wr, +64) for
// instance columns [16 wc, +16), reduces q2 . gelu over its 64 rows with warp
// shuffles, and adds its 16 partial sums into y with global atomics (y zeroed
// before the launch; the wr = 0 warp adds c2 with its partial).  Each output
// then receives exactly two additions onto zero, (c2 + part_0) and part_1,
// and x + y = y + x holds exactly, so the result does not depend on their
// order.
constexpr int kRoHid = 128;

template <int ST> struct RoLayout {
    static constexpr int kWarps = 8;
    static constexpr int kThreads = 32 * (kWarps + 1);
    static constexpr int kTile = kCmC * kCmBN * 2;  // 8 KB
    static constexpr int kWP = kCmC + 8;
    static constexpr int kW = kRoHid * kWP * 2;     // 18 KB
    static constexpr size_t kWOff = (size_t)ST * kTile;
    static constexpr size_t kBytes = kWOff + kW;
    static constexpr size_t kAlloc = kBytes + 1024;
};

template <typename E, int ST, int MINB>
__global__ void __launch_bounds__(RoLayout<ST>::kThreads, MINB)
ro_ws_kernel(const __grid_constant__ CUtensorMap tH, const float *__restrict__ Q1,
             const float *__restrict__ c1, const float *__restrict__ q2,
             const float *__restrict__ c2, float *__restrict__ y, int Bp, int nb,
             long long total, long long wait_limit, unsigned int *__restrict__ status)
{
    using L = RoLayout<ST>;
    constexpr int FM = 4;  // 64 rows per warp
    extern __shared__ unsigned char ro_smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(ro_smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[ST], empty[ST];
    E *sW = reinterpret_cast<E *>(smem + L::kWOff);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < ST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], L::kWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = tid; e < kRoHid * kCmC; e += L::kThreads) {
        const int m = e / kCmC, k = e % kCmC;
        sW[m * L::kWP + k] = Elem<E>::cvt(Q1[e]);
    }
    __syncthreads();

    if (warp == L::kWarps) {
        if (lane != 0) return;
        long long it = 0;
        for (long long i = blockIdx.x; i < total; i += gridDim.x, it++) {
            const int s = (int)(it % ST);
            if (it >= ST &&
                !mbar_wait_bounded(&empty[s], (uint32_t)(((it / ST) - 1) & 1), wait_limit)) {
                atomicOr(status, kStatusTimeout);
                for (long long j = it - ST + 1; j < it; j++)
                    (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), wait_limit);
                return;
            }
            const int p = (int)(i / nb), b0 = (int)(i % nb) * kCmBN;
            mbar_expect_tx(&full[s], (uint32_t)L::kTile);
            tma_load_2d(smem + (size_t)s * L::kTile, &tH, b0, p * kCmC, &full[s]);
        }
        return;
    }

    const int g = lane >> 2, t = lane & 3;
    const int col0 = (warp & 3) * 16, row0 = (warp >> 2) * 64;
    float cm[FM][2], qm[FM][2];
#pragma unroll
    for (int fm = 0; fm < FM; fm++)
#pragma unroll
        for (int hh = 0; hh < 2; hh++) {
            cm[fm][hh] = c1[row0 + 16 * fm + g + 8 * hh];
            qm[fm][hh] = q2[row0 + 16 * fm + g + 8 * hh];
        }
    const float cadd = row0 == 0 ? c2[0] : 0.f;
    long long it = 0;
    for (long long i = blockIdx.x; i < total; i += gridDim.x, it++) {
        const int s = (int)(it % ST);
        if (!mbar_wait_bounded(&full[s], (uint32_t)((it / ST) & 1), wait_limit)) {
            atomicOr(status, kStatusTimeout);
            for (long long j = it + 1; j < it + ST && j < total; j++)
                (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), wait_limit);
            return;
        }
        const unsigned char *sB = smem + (size_t)s * L::kTile;
        float acc[FM][2][4];
#pragma unroll
        for (int fm = 0; fm < FM; fm++)
#pragma unroll
            for (int fn = 0; fn < 2; fn++)
#pragma unroll
                for (int r = 0; r < 4; r++) acc[fm][fn][r] = 0.f;
#pragma unroll
        for (int kk = 0; kk < kCmC; kk += 16) {
            uint32_t a[FM][4], b[4];
#pragma unroll
            for (int fm = 0; fm < FM; fm++)
                ldsm_x4(a[fm], sW + (row0 + 16 * fm + (lane & 15)) * L::kWP + kk + (lane >> 4) * 8);
            const int krow = kk + (lane & 15);
            const int chunk = (col0 >> 3) + (lane >> 4);
            ldsm_x4_t(b, sB + krow * 128 + ((chunk ^ (krow & 7)) << 4));
#pragma unroll
            for (int fm = 0; fm < FM; fm++) {
                mma16816<E>(acc[fm][0], a[fm], b[0], b[1]);
                mma16816<E>(acc[fm][1], a[fm], b[2], b[3]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);  // the tile is in registers now
        // part += q2 gelu(acc + c1) on column pairs, in FP32x2 instructions
        float2 part[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int fm = 0; fm < FM; fm++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++)
#pragma unroll
                for (int fn = 0; fn < 2; fn++) {
                    const float2 u =
                        __fadd2_rn(make_float2(acc[fm][fn][2 * hh], acc[fm][fn][2 * hh + 1]),
                                   make_float2(cm[fm][hh], cm[fm][hh]));
                    part[fn] = __ffma2_rn(make_float2(qm[fm][hh], qm[fm][hh]), gelu2_f(u), part[fn]);
                }
#pragma unroll
        for (int fn = 0; fn < 2; fn++)
#pragma unroll
            for (int c = 0; c < 2; c++) {
                float v = c ? part[fn].y : part[fn].x;
                v += __shfl_xor_sync(0xffffffffu, v, 4);
                v += __shfl_xor_sync(0xffffffffu, v, 8);
                v += __shfl_xor_sync(0xffffffffu, v, 16);
                if (c)
                    part[fn].y = v;
                else
                    part[fn].x = v;
            }
        if (g == 0) {
            const int p = (int)(i / nb), b0 = (int)(i % nb) * kCmBN;
            float *yrow = y + (long long)p * Bp + b0 + col0;
#pragma unroll
            for (int fn = 0; fn < 2; fn++) {
                atomicAdd(yrow + 8 * fn + 2 * t, part[fn].x + cadd);
                atomicAdd(yrow + 8 * fn + 2 * t + 1, part[fn].y + cadd);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The axis-k transforms of an inference pass, the same warp-specialised
// structure.  Both are small real products per slab s = (i, j) of the grid:
//   forward  T1[s][r][cb] = sum_k A[r][k] h[s N + k][cb],  A = [Re F; Im F]
//            (24 x 32 at 12 modes, N = 32: complex F times the real h),
//   inverse  S[s N + k][cb] = sum_q A[k][q] U2[s][q][cb],  A = [Re G, -Im G]
//            (the real part of complex G times complex U2),
// with cb running over channels x instances (64-column blocks).  One work item
// is one slab and two column blocks.  The 32 x 32 A (zero padded, laid out so
// that the K blocks of 16 hold the same terms as in the general kernel: real
// parts in K rows 0..15, imaginary parts in 16..31) stays in shared memory;
// the producer loads the item's B rows with 2D TMA copies (one per column block
// and K half when the input is split), eight consumer warps each multiply a
// 32 x 16 block and store its first out_rows rows with a 2D TMA store.
template <int ST> struct AxLayout {
    static constexpr int kWarps = 8;
    static constexpr int kThreads = 32 * (kWarps + 1);
    static constexpr int kTile = 32 * 128;           // 32 K rows x 64 columns, 16-bit
    static constexpr int kStage = 2 * kTile;         // two column blocks
    static constexpr int kAP = 32 + 8;
    static constexpr int kA = 32 * kAP * 2;
    static constexpr int kStg = 32 * 16 * 2;         // 32 rows x 16 columns
    static constexpr size_t kAOff = (size_t)ST * kStage;
    static constexpr size_t kStgOff = kAOff + kA;
    static constexpr size_t kBytes = kStgOff + (size_t)kWarps * 2 * kStg;
    static constexpr size_t kAlloc = kBytes + 1024;
};

struct AxArgs {
    const float *A;   // 32 x 32 FP32, row-major, already in the K layout above
    int nb;           // 64-column blocks per slab row (even)
    long long total;  // work items: slabs x nb / 2
    int ld_rows;      // rows of one TMA load (= the box height of tB)
    int split;        // 0: one load into K rows 0..ld_rows-1; 1: rows 0.. and 16..
    int in_rows;      // input rows per slab
    int out_rows;     // output rows per slab (= the box height of tC)
};

template <typename E, int ST, int MINB>
__global__ void __launch_bounds__(AxLayout<ST>::kThreads, MINB)
ax_ws_kernel(const __grid_constant__ CUtensorMap tB, const __grid_constant__ CUtensorMap tC,
             const AxArgs a, long long wait_limit, unsigned int *__restrict__ status)
{
    using L = AxLayout<ST>;
    using T2 = typename Elem<E>::T2;
    extern __shared__ unsigned char ax_smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(ax_smem_raw) + 1023) & ~(uintptr_t)1023);
    __shared__ uint64_t full[ST], empty[ST];
    E *sA = reinterpret_cast<E *>(smem + L::kAOff);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid == 0) {
        for (int s = 0; s < ST; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], L::kWarps);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int e = tid; e < 32 * 32; e += L::kThreads)
        sA[(e / 32) * L::kAP + (e % 32)] = Elem<E>::cvt(a.A[e]);
    // K rows that no load writes stay zero (their A columns are zero too)
    for (int e = tid; e < ST * L::kStage / 16; e += L::kThreads)
        reinterpret_cast<uint4 *>(smem)[e] = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();

    if (warp == L::kWarps) {
        if (lane != 0) return;
        const uint32_t bytes = (uint32_t)(2 * (a.split ? 2 : 1) * a.ld_rows * 128);
        long long it = 0;
        for (long long i = blockIdx.x; i < a.total; i += gridDim.x, it++) {
            const int s = (int)(it % ST);
            if (it >= ST &&
                !mbar_wait_bounded(&empty[s], (uint32_t)(((it / ST) - 1) & 1), wait_limit)) {
                atomicOr(status, kStatusTimeout);
                for (long long j = it - ST + 1; j < it; j++)
                    (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), wait_limit);
                return;
            }
            const int half = a.nb / 2;
            const int slab = (int)(i / half), b0 = (int)(i % half) * 128;
            unsigned char *st = smem + (size_t)s * L::kStage;
            mbar_expect_tx(&full[s], bytes);
            for (int cb = 0; cb < 2; cb++) {
                tma_load_2d(st + cb * L::kTile, &tB, b0 + 64 * cb, slab * a.in_rows, &full[s]);
                if (a.split)
                    tma_load_2d(st + cb * L::kTile + 16 * 128, &tB, b0 + 64 * cb,
                                slab * a.in_rows + a.ld_rows, &full[s]);
            }
        }
        return;
    }

    const int g = lane >> 2, t = lane & 3;
    const int cb = warp >> 2, col0 = (warp & 3) * 16;
    E *stg0 = reinterpret_cast<E *>(smem + L::kStgOff + (size_t)warp * 2 * L::kStg);
    long long it = 0;
    for (long long i = blockIdx.x; i < a.total; i += gridDim.x, it++) {
        const int s = (int)(it % ST);
        if (!mbar_wait_bounded(&full[s], (uint32_t)((it / ST) & 1), wait_limit)) {
            atomicOr(status, kStatusTimeout);
            for (long long j = it + 1; j < it + ST && j < a.total; j++)
                (void)mbar_wait_bounded(&full[j % ST], (uint32_t)((j / ST) & 1), wait_limit);
            if (lane == 0) bulk_wait_all();
            return;
        }
        const unsigned char *sB = smem + (size_t)s * L::kStage + cb * L::kTile;
        float acc[2][2][4];
#pragma unroll
        for (int fm = 0; fm < 2; fm++)
#pragma unroll
            for (int fn = 0; fn < 2; fn++)
#pragma unroll
                for (int r = 0; r < 4; r++) acc[fm][fn][r] = 0.f;
#pragma unroll
        for (int kk = 0; kk < 32; kk += 16) {
            uint32_t af[2][4], b[4];
#pragma unroll
            for (int fm = 0; fm < 2; fm++)
                ldsm_x4(af[fm], sA + (16 * fm + (lane & 15)) * L::kAP + kk + (lane >> 4) * 8);
            const int krow = kk + (lane & 15);
            const int chunk = (col0 >> 3) + (lane >> 4);
            ldsm_x4_t(b, sB + krow * 128 + ((chunk ^ (krow & 7)) << 4));
#pragma unroll
            for (int fm = 0; fm < 2; fm++) {
                mma16816<E>(acc[fm][0], af[fm], b[0], b[1]);
                mma16816<E>(acc[fm][1], af[fm], b[2], b[3]);
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
        E *stg = stg0 + (it & 1) * (32 * 16);
        if (lane == 0) bulk_wait_read1();
        __syncwarp();
#pragma unroll
        for (int fm = 0; fm < 2; fm++)
#pragma unroll
            for (int hh = 0; hh < 2; hh++) {
                const int m = 16 * fm + g + 8 * hh;
#pragma unroll
                for (int fn = 0; fn < 2; fn++)
                    *reinterpret_cast<T2 *>(stg + m * 16 + 8 * fn + 2 * t) =
                        Elem<E>::cvt2(acc[fm][fn][2 * hh], acc[fm][fn][2 * hh + 1]);
            }
        fence_async_smem();
        __syncwarp();
        if (lane == 0) {
            const int half = a.nb / 2;
            const int slab = (int)(i / half), b0 = (int)(i % half) * 128;
            tma_store_2d(&tC, stg, b0 + 64 * cb + col0, slab * a.out_rows);
            bulk_commit();
        }
    }
    if (lane == 0) bulk_wait_all();
}

}  // namespace fno
}  // namespace sbte
