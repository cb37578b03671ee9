// fno_gemm.cuh -- the BF16 tensor-core GEMMs of the learned collision
// operator (FP32 accumulation).
//
// Every product in the network is one of two shapes once activations sit in
// the layout [point][channel][instance] (instance index innermost):
//
//  * gemm_sa ("small A, streamed B"):  C[m][n] = sum_k A[m][k] B[k][n] with
//    A a small dense matrix (a DFT axis matrix, a channel-mixing matrix;
//    M, K <= 128) and B a long stream (N up to 10^8) contiguous along n.
//    A is read once per CTA from FP32 and rounded to BF16 in shared memory;
//    B tiles stream through a two-stage cp.async pipeline.
//  * gemm_nt ("weight gradient"):  C[m][n] += sum_k A[m][k] B[n][k] with
//    both operands contiguous along k and K huge; K is split over CTAs and
//    the FP32 partial products are added atomically.
//
// Operand views.  A streamed operand element (r, n) (r = the k row of B, or
// the m row of C) sits at
//     base + r * s_r + (n / w) * s_blk + (n % w)           (+ im for Im)
// i.e. n runs over blocks of w contiguous elements (w a multiple of 8).
// Complex tensors store the real and imaginary parts as two such views im
// elements apart.  Batches: z -> (z / nz2) * s_z1 + (z % nz2) * s_z2.
// n / w is evaluated with a multiply-high by a magic number precomputed on
// the host (division by an invariant integer, Granlund and Montgomery
// 1994), on 32-bit n: a 64-bit integer division costs tens of instructions
// per 16-byte chunk and made these kernels issue-bound.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

namespace sbte {
namespace fno {

using bf16 = __nv_bfloat16;
using f16 = __half;

// The 16-bit element type of a network: BF16 or FP16 (same tensor-core rate;
// FP16 keeps 3 more mantissa bits, BF16 the FP32 exponent range).
template <typename E> struct Elem;
template <> struct Elem<bf16> {
    using T2 = __nv_bfloat162;
    static __device__ __forceinline__ bf16 cvt(float x) { return __float2bfloat16_rn(x); }
    static __device__ __forceinline__ T2 cvt2(float a, float b) { return __floats2bfloat162_rn(a, b); }
    static __device__ __forceinline__ float2 f2(T2 v) { return __bfloat1622float2(v); }
};
template <> struct Elem<f16> {
    using T2 = __half2;
    static __device__ __forceinline__ f16 cvt(float x) { return __float2half_rn(x); }
    static __device__ __forceinline__ T2 cvt2(float a, float b) { return __floats2half2_rn(a, b); }
    static __device__ __forceinline__ float2 f2(T2 v) { return __half22float2(v); }
};

struct StreamView {
    const void *p;
    long long s_r, s_blk, w, im, s_z1, s_z2;
    unsigned wm, ws;  // n / w = (umulhi(n, wm) + n) >> ws   (set by fastdiv_init)
};

// Magic multiplier and shift for unsigned 32-bit division by d >= 1:
// s = ceil(log2 d), m = floor(2^32 (2^s - d) / d) + 1; then for every
// 32-bit n, n / d = (umulhi(n, m) + n) >> s, the sum taken in 64 bits.
inline void fastdiv_init(unsigned d, unsigned &m, unsigned &s)
{
    s = 0;
    while ((1ull << s) < d) s++;
    m = (unsigned)(((1ull << 32) * ((1ull << s) - d)) / d + 1);
}
__device__ __forceinline__ unsigned fastdiv(unsigned n, unsigned m, unsigned s)
{
    return (unsigned)(((unsigned long long)__umulhi(n, m) + n) >> s);
}

enum Epi : int {
    kEpiBF16 = 0,     // real output, BF16 store
    kEpiCplxBF16 = 1, // complex output (re at off, im at off + im), BF16 store
    kEpiF32 = 2,      // real output, FP32 store
    kEpiAccF32 = 3,   // real output, FP32 C += result
    kEpiLayer = 4,    // z = acc + bias[m] + addend; zst = z; hout = act(z)
    kEpiProj = 5,     // y[n] = c2 + sum_m q2[m] gelu(acc[m][n] + c1[m]); ust = acc + c1
};

struct SaArgs {
    // A(m, k) = A[a_off + m * sAm + k * sAk] (+ imA for Im), FP32
    const float *A;
    long long sAm, sAk, imA;
    float a_im_sign;       // -1 applies conj(A)
    const int *a_tab;      // optional: a_off = a_tab[z] * s_atab
    long long s_atab;
    int M, K, KP;          // KP: K rounded up to 16
    StreamView B;          // B(k, n)
    StreamView C;          // C(m, n)
    long long Nn;          // n extent (multiple of 8)
    int nz, nz2;
    // epilogue operands
    const float *bias;     // kEpiLayer
    const void *addend;    // kEpiLayer: 16-bit elements, same view as C
    float *zst;            // kEpiLayer / kEpiProj: optional FP32 store, same view as C
    void *hout;            // kEpiLayer: 16-bit store, same view as C
    float alpha;           // kEpiAccF32: C += alpha * result
    int act;               // kEpiLayer: 1 = GELU
    const float *c1, *q2;  // kEpiProj
    const float *c2;       // kEpiProj: one value on the device
    float *y;              // kEpiProj: y[n]
    int bil;               // kEpiProj: bilinear readout over row pairs (m, m + 8)
    // host-side bounds check: element counts of A, B, C (and of the
    // epilogue arrays that share C's view); 0 skips the check
    long long extA, extB, extC;
    int a_tab_max;  // largest value in a_tab (host-side bounds check)
    // 1: each CTA runs one contiguous range of work items instead of every
    // gridDim-th item, so that a per-batch A (a_tab) is reloaded only when the
    // batch changes, not on every item
    int contig;
};

struct NtArgs {
    // A(m, k) = A[zA + m * a_m + (k / a_w) * a_blk + k % a_w]; same for B(n, k)
    const void *A;
    long long a_m, a_blk, a_w, a_z1, a_z2;
    const void *B;
    long long b_n, b_blk, b_w, b_z1, b_z2;
    float *C;              // C[c_tab ? c_tab[z] * c_tabs : 0 + m * c_m + n]
    long long c_m;
    const int *c_tab;
    long long c_tabs;
    int M, N;
    long long K, KC;       // K and the per-CTA chunk (multiples of 32)
    int nz, nz2;
    float alpha;
    long long extA, extB, extC;  // host-side bounds check (element counts)
    unsigned awm, aws, bwm, bws;  // fast division by a_w and b_w (fastdiv_init)
};

// erf by Abramowitz and Stegun 7.1.26 (Hastings' rational approximation):
// erf(x) = 1 - t (a1 + t (a2 + t (a3 + t (a4 + t a5)))) e^{-x^2},
// t = 1 / (1 + p x), x >= 0, odd extension; |error| <= 1.5e-7 in exact
// arithmetic and 6.1e-7 evaluated in FP32 on [-12, 12] (tests check the
// constants against scipy's erf); the error is far below the 16-bit
// resolution of the activations.  The training backward's GELU derivative
// uses it.
__device__ __forceinline__ float erf_as(float x)
{
    const float ax = fabsf(x);
    const float t = __frcp_rn(fmaf(0.3275911f, ax, 1.0f));
    const float poly =
        fmaf(fmaf(fmaf(fmaf(1.061405429f, t, -1.453152027f), t, 1.421413741f), t, -0.284496736f),
             t, 0.254829592f) * t;
    const float r = fmaf(-poly, __expf(-ax * ax), 1.0f);
    return copysignf(r, x);
}
// The forward GELU, z Phi(z) = 0.5 z (1 + erf(z / sqrt 2)), written with the
// same rational approximation in its erfc form: for u = |z| / sqrt 2,
//   erfc(u) = t (a1 + t (a2 + ...)) e^{-u^2},   t = 1 / (1 + p u),
//   GELU(z) = max(z, 0) - |z| (erfc(u) / 2)
// (z >= 0: z - z erfc / 2; z < 0: z erfc / 2).  The coefficients are halved
// (exact in binary), the reciprocal and 2^x are the single PTX approximations
// (rcp.approx, ex2.approx; relative error about 1 ulp), and the tail needs no
// cancellation 1 - erf for negative z.  About a dozen instructions, two of
// them on the transcendental unit.  gelu2_f does two lanes with FP32x2
// instructions in the same order, so its lanes equal gelu_f bit for bit.
namespace gelu_c {
constexpr float kInvSqrt2 = 0.70710678118654752f;
constexpr float kP = 0.3275911f;
constexpr float kH1 = 0.5f * 0.254829592f, kH2 = 0.5f * -0.284496736f,
                kH3 = 0.5f * 1.421413741f, kH4 = 0.5f * -1.453152027f,
                kH5 = 0.5f * 1.061405429f;
constexpr float kNegLog2e = -1.4426950408889634f;
}  // namespace gelu_c
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ float gelu_f(float z)
{
    using namespace gelu_c;
    const float a = fabsf(z);
    const float u = a * kInvSqrt2;
    const float t = rcp_approx(fmaf(u, kP, 1.0f));
    float h = fmaf(kH5, t, kH4);
    h = fmaf(h, t, kH3);
    h = fmaf(h, t, kH2);
    h = fmaf(h, t, kH1);
    h = h * t;
    const float e = ex2_approx(u * (u * kNegLog2e));
    return fmaf(-a, h * e, fmaxf(z, 0.0f));
}
__device__ __forceinline__ float2 gelu2_f(float2 z)
{
    using namespace gelu_c;
    const float2 a = make_float2(fabsf(z.x), fabsf(z.y));
    const float2 u = __fmul2_rn(a, make_float2(kInvSqrt2, kInvSqrt2));
    const float2 d = __ffma2_rn(u, make_float2(kP, kP), make_float2(1.0f, 1.0f));
    const float2 t = make_float2(rcp_approx(d.x), rcp_approx(d.y));
    float2 h = __ffma2_rn(make_float2(kH5, kH5), t, make_float2(kH4, kH4));
    h = __ffma2_rn(h, t, make_float2(kH3, kH3));
    h = __ffma2_rn(h, t, make_float2(kH2, kH2));
    h = __ffma2_rn(h, t, make_float2(kH1, kH1));
    h = __fmul2_rn(h, t);
    const float2 m = __fmul2_rn(u, __fmul2_rn(u, make_float2(kNegLog2e, kNegLog2e)));
    const float2 he = __fmul2_rn(h, make_float2(ex2_approx(m.x), ex2_approx(m.y)));
    return __ffma2_rn(make_float2(-a.x, -a.y), he, make_float2(fmaxf(z.x, 0.0f), fmaxf(z.y, 0.0f)));
}
__device__ __forceinline__ float gelu_grad(float x)
{
    return 0.5f * (1.0f + erf_as(x * 0.70710678118654752f)) +
           x * 0.39894228040143268f * __expf(-0.5f * x * x);
}

__device__ __forceinline__ uint32_t smem_addr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void cp_async16(void *sdst, const void *gsrc, bool valid)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_addr(sdst)),
                 "l"(gsrc), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N> __device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const void *p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_addr(p)));
}
template <typename E>
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1)
{
    if constexpr (std::is_same<E, f16>::value)
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, "
            "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
    else
        asm volatile(
            "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
            "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
            : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ long long view_off(const StreamView &v, long long r, long long n)
{
    const unsigned nn = (unsigned)n;
    const unsigned q = fastdiv(nn, v.wm, v.ws);
    return r * v.s_r + (long long)q * v.s_blk + (long long)(nn - q * (unsigned)v.w);
}
__device__ __forceinline__ long long zoff(long long z, int nz2, long long s1, long long s2)
{
    const unsigned q = (unsigned)z / (unsigned)nz2;  // z < 2^31 (checked on the host)
    return (long long)q * s1 + (long long)((unsigned)z - q * (unsigned)nz2) * s2;
}

// ------------------------------------------------------------ gemm_sa ---
// MT x BN output tile per work item; WM x WN warps; AC / BC: A / B complex;
// an ST-stage cp.async ring over the work items (ST - 1 tiles in flight).
// Complex output (kEpiCplxBF16) holds re and im accumulators; a complex x
// complex product with a real epilogue keeps only the real part.  16-bit
// outputs go through a shared-memory tile and leave as 16-byte vectors; the
// layer epilogue's addend streams in with the B tile, and its tile slot then
// stages the layer output.
template <int MT, int BN, int WM, bool AC, bool BC, int EPI, int ST> struct SaLayout {
    static constexpr int kParts = BC ? 2 : 1;
    static constexpr bool kAdd = EPI == kEpiLayer;
    static constexpr bool kOwnStage = EPI == kEpiBF16 || EPI == kEpiCplxBF16;
    static constexpr int kBP = BN + 8;
    static constexpr int kStageRows = kOwnStage ? (EPI == kEpiCplxBF16 ? 2 : 1) * MT : 0;
    // elements of one ring stage for K rounded to KP
    static __host__ __device__ int stage_elems(int KP) { return kParts * KP * kBP + (kAdd ? MT * kBP : 0); }
    static __host__ __device__ size_t bytes(int KP)
    {
        return 2 * ((size_t)(AC ? 3 : 1) * MT * (KP + 8) + (size_t)ST * stage_elems(KP) +
                    (size_t)kStageRows * kBP) +
               (EPI == kEpiProj ? (size_t)WM * BN * 4 : 0);
    }
};

template <typename E, int MT, int BN, int WM, int WN, bool AC, bool BC, int EPI, int ST>
__global__ void __launch_bounds__(WM *WN * 32) gemm_sa_kernel(const SaArgs a)
{
    using T2 = typename Elem<E>::T2;
    using L = SaLayout<MT, BN, WM, AC, BC, EPI, ST>;
    constexpr int NTH = WM * WN * 32;
    constexpr int WR = MT / WM, WC = BN / WN;
    constexpr int FM = WR / 16, FN = WC / 8;
    static_assert(WR % 16 == 0 && WC % 16 == 0, "warp tile");
    constexpr bool CO = (EPI == kEpiCplxBF16);
    constexpr bool IM = CO || (AC && !BC);  // imaginary accumulator needed
    static_assert(!(AC && !BC) || CO, "complex A x real B gives a complex result");
    constexpr int PARTS = L::kParts, BP = L::kBP, CH = BN / 8;
    constexpr bool STG = L::kOwnStage || L::kAdd;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int KP = a.KP, ap = KP + 8;
    E *sAr = reinterpret_cast<E *>(smem_raw);
    E *sAi = sAr + MT * ap;
    E *sAn = sAi + MT * ap;
    E *ring = sAr + (AC ? 3 : 1) * MT * ap;
    const int tileB = KP * BP;
    const int stageE = L::stage_elems(KP);
    E *own = ring + ST * stageE;  // output staging tile (kOwnStage)
    float *red = reinterpret_cast<float *>(own + L::kStageRows * BP);  // kEpiProj: [WM][BN]

    const unsigned ntiles = (unsigned)((a.Nn + BN - 1) / BN);
    const unsigned total = ntiles * (unsigned)a.nz;
    const unsigned chunk = (total + gridDim.x - 1) / gridDim.x;
    const unsigned step = a.contig ? 1u : gridDim.x;
    unsigned item = a.contig ? blockIdx.x * chunk : blockIdx.x;
    const unsigned end = a.contig ? min(total, item + chunk) : total;
    if (item >= end) return;

    const E *Bb = static_cast<const E *>(a.B.p);
    auto issue = [&](unsigned it, int stage) {
        const unsigned z = it / ntiles;
        const long long n0 = (long long)(it - z * ntiles) * BN;
        const long long zb = zoff(z, a.nz2, a.B.s_z1, a.B.s_z2);
        E *base = ring + stage * stageE;
        for (int c = threadIdx.x; c < KP * CH; c += NTH) {
            const int r = c / CH, cn = c % CH;
            const long long n = n0 + cn * 8;
            const bool ok = (r < a.K) && (n < a.Nn);
            const long long off = ok ? zb + view_off(a.B, r, n) : 0;
#pragma unroll
            for (int part = 0; part < PARTS; part++)
                cp_async16(base + part * tileB + r * BP + cn * 8, Bb + off + (part ? a.B.im : 0),
                           ok);
        }
        if constexpr (L::kAdd) {
            const long long zc = zoff(z, a.nz2, a.C.s_z1, a.C.s_z2);
            const E *ad = static_cast<const E *>(a.addend);
            E *sa = base + PARTS * tileB;
            for (int c = threadIdx.x; c < MT * CH; c += NTH) {
                const int r = c / CH, cn = c % CH;
                const long long n = n0 + cn * 8;
                const bool ok = (r < a.M) && (n < a.Nn);
                const long long off = ok ? zc + view_off(a.C, r, n) : 0;
                cp_async16(sa + r * BP + cn * 8, ad + off, ok);
            }
        }
    };

#pragma unroll
    for (int s = 0; s < ST - 1; s++) {
        const unsigned it = item + (unsigned)s * step;
        if (it < end) issue(it, s);
        cp_async_commit();
    }

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = warp / WN, wn = warp % WN;
    const int g = lane >> 2, t = lane & 3;
    long long cur_z = -1;
    int stage = 0;
    for (; item < end; item += step) {
        const unsigned pre = item + (unsigned)(ST - 1) * step;
        if (pre < end) issue(pre, (stage + ST - 1) % ST);
        cp_async_commit();
        const unsigned z = item / ntiles;
        const long long n0 = (long long)(item - z * ntiles) * BN;
        if (cur_z < 0 || (a.a_tab && (long long)z != cur_z)) {
            __syncthreads();
            const long long aoff = a.a_tab ? (long long)a.a_tab[z] * a.s_atab : 0;
            for (int e = threadIdx.x; e < MT * KP; e += NTH) {
                const int m = e / KP, k = e % KP;
                float re = 0.f, im = 0.f;
                if (m < a.M && k < a.K) {
                    const float *src = a.A + aoff + m * a.sAm + k * a.sAk;
                    re = src[0];
                    if (AC) im = a.a_im_sign * src[a.imA];
                }
                sAr[m * ap + k] = Elem<E>::cvt(re);
                if (AC) {
                    sAi[m * ap + k] = Elem<E>::cvt(im);
                    sAn[m * ap + k] = Elem<E>::cvt(-im);
                }
            }
            cur_z = z;
        }
        cp_async_wait<ST - 1>();
        __syncthreads();

        float accR[FM][FN][4], accI[IM ? FM : 1][IM ? FN : 1][4];
#pragma unroll
        for (int i = 0; i < FM; i++)
#pragma unroll
            for (int j = 0; j < FN; j++)
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    accR[i][j][r] = 0.f;
                    if (IM) accI[IM ? i : 0][IM ? j : 0][r] = 0.f;
                }
        E *sbase = ring + stage * stageE;
        const E *sBr = sbase;
        const E *sBi = sBr + tileB;
        for (int kk = 0; kk < KP; kk += 16) {
            uint32_t ar[FM][4], ai[AC ? FM : 1][4], an[AC ? FM : 1][4];
#pragma unroll
            for (int fm = 0; fm < FM; fm++) {
                const int row = wm * WR + fm * 16 + (lane & 15);
                const int col = kk + (lane >> 4) * 8;
                ldsm_x4(ar[fm], sAr + row * ap + col);
                if (AC) {
                    ldsm_x4(ai[AC ? fm : 0], sAi + row * ap + col);
                    if (BC) ldsm_x4(an[AC ? fm : 0], sAn + row * ap + col);
                }
            }
#pragma unroll
            for (int f2 = 0; f2 < FN / 2; f2++) {
                uint32_t br[4], bi[4];
                const int krow = kk + (lane & 15);
                const int ncol = wn * WC + f2 * 16 + (lane >> 4) * 8;
                ldsm_x4_t(br, sBr + krow * BP + ncol);
                if (BC) ldsm_x4_t(bi, sBi + krow * BP + ncol);
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int fn = f2 * 2 + h;
#pragma unroll
                    for (int fm = 0; fm < FM; fm++) {
                        if (!AC) {
                            mma16816<E>(accR[fm][fn], ar[fm], br[2 * h], br[2 * h + 1]);
                        } else if (!BC) {
                            mma16816<E>(accR[fm][fn], ar[fm], br[2 * h], br[2 * h + 1]);
                            mma16816<E>(accI[IM ? fm : 0][IM ? fn : 0], ai[AC ? fm : 0],
                                        br[2 * h], br[2 * h + 1]);
                        } else {
                            mma16816<E>(accR[fm][fn], ar[fm], br[2 * h], br[2 * h + 1]);
                            mma16816<E>(accR[fm][fn], an[AC ? fm : 0], bi[2 * h], bi[2 * h + 1]);
                            if (CO) {
                                mma16816<E>(accI[IM ? fm : 0][IM ? fn : 0], ar[fm], bi[2 * h],
                                            bi[2 * h + 1]);
                                mma16816<E>(accI[IM ? fm : 0][IM ? fn : 0], ai[AC ? fm : 0],
                                            br[2 * h], br[2 * h + 1]);
                            }
                        }
                    }
                }
            }
        }

        // ---- epilogue
        const long long zc = zoff(z, a.nz2, a.C.s_z1, a.C.s_z2);
        if constexpr (EPI == kEpiProj) {
            float part[FN][2];
#pragma unroll
            for (int fn = 0; fn < FN; fn++) part[fn][0] = part[fn][1] = 0.f;
#pragma unroll
            for (int fm = 0; fm < FM; fm++) {
                const int m = wm * WR + fm * 16 + g;   // rows m and m + 8 of this thread
                if (m >= a.M) continue;
                if (a.bil) {
                    // pair e = 8 (m / 16) + m % 8: left factor row m, right factor row m + 8
                    const float cl = a.c1[m], cr = a.c1[m + 8];
                    const float q = a.q2[(m >> 4) * 8 + (m & 7)];
#pragma unroll
                    for (int fn = 0; fn < FN; fn++) {
                        const long long n = n0 + wn * WC + fn * 8 + 2 * t;
                        const float l0 = accR[fm][fn][0] + cl, l1 = accR[fm][fn][1] + cl;
                        const float r0 = accR[fm][fn][2] + cr, r1 = accR[fm][fn][3] + cr;
                        if (a.zst && n < a.Nn) {
                            *reinterpret_cast<float2 *>(a.zst + zc + view_off(a.C, m, n)) =
                                make_float2(l0, l1);
                            *reinterpret_cast<float2 *>(a.zst + zc + view_off(a.C, m + 8, n)) =
                                make_float2(r0, r1);
                        }
                        part[fn][0] += q * l0 * r0;
                        part[fn][1] += q * l1 * r1;
                    }
                    continue;
                }
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int mh = m + hh * 8;
                    if (mh >= a.M) continue;
                    const float c1 = a.c1[mh], q2 = a.q2[mh];
#pragma unroll
                    for (int fn = 0; fn < FN; fn++) {
                        const long long n = n0 + wn * WC + fn * 8 + 2 * t;
                        const float u0 = accR[fm][fn][2 * hh] + c1;
                        const float u1 = accR[fm][fn][2 * hh + 1] + c1;
                        if (a.zst && n < a.Nn) {
                            float *dst = a.zst + zc + view_off(a.C, mh, n);
                            *reinterpret_cast<float2 *>(dst) = make_float2(u0, u1);
                        }
                        part[fn][0] += q2 * gelu_f(u0);
                        part[fn][1] += q2 * gelu_f(u1);
                    }
                }
            }
#pragma unroll
            for (int fn = 0; fn < FN; fn++)
#pragma unroll
                for (int c = 0; c < 2; c++) {
                    float v = part[fn][c];
                    v += __shfl_xor_sync(0xffffffffu, v, 4);
                    v += __shfl_xor_sync(0xffffffffu, v, 8);
                    v += __shfl_xor_sync(0xffffffffu, v, 16);
                    part[fn][c] = v;
                }
            if (g == 0) {
#pragma unroll
                for (int fn = 0; fn < FN; fn++) {
                    red[wm * BN + wn * WC + fn * 8 + 2 * t] = part[fn][0];
                    red[wm * BN + wn * WC + fn * 8 + 2 * t + 1] = part[fn][1];
                }
            }
            __syncthreads();
            for (int c = threadIdx.x; c < BN; c += NTH) {
                const long long n = n0 + c;
                if (n < a.Nn) {
                    float s = a.c2[0];
#pragma unroll
                    for (int w = 0; w < WM; w++) s += red[w * BN + c];
                    a.y[n] = s;
                }
            }
        } else if constexpr (STG) {
            // values into the staging tile (rows: re then im for complex output)
            E *tile = L::kAdd ? sbase + PARTS * tileB : own;
#pragma unroll
            for (int fm = 0; fm < FM; fm++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int m = wm * WR + fm * 16 + g + hh * 8;
#pragma unroll
                    for (int fn = 0; fn < FN; fn++) {
                        const int col = wn * WC + fn * 8 + 2 * t;
                        const float v0 = accR[fm][fn][2 * hh], v1 = accR[fm][fn][2 * hh + 1];
                        T2 *dst = reinterpret_cast<T2 *>(tile + m * BP + col);
                        if constexpr (L::kAdd) {
                            const long long n = n0 + col;
                            const float bm = m < a.M ? a.bias[m] : 0.f;
                            const float2 ad = Elem<E>::f2(*dst);
                            const float z0 = v0 + bm + ad.x, z1 = v1 + bm + ad.y;
                            if (a.zst && m < a.M && n < a.Nn)
                                *reinterpret_cast<float2 *>(a.zst + zc + view_off(a.C, m, n)) =
                                    make_float2(z0, z1);
                            if (a.act) {
                                const float2 o = gelu2_f(make_float2(z0, z1));
                                *dst = Elem<E>::cvt2(o.x, o.y);
                            } else {
                                *dst = Elem<E>::cvt2(z0, z1);
                            }
                        } else {
                            *dst = Elem<E>::cvt2(v0, v1);
                            if constexpr (CO)
                                *reinterpret_cast<T2 *>(tile + (MT + m) * BP + col) =
                                    Elem<E>::cvt2(accI[IM ? fm : 0][IM ? fn : 0][2 * hh],
                                                  accI[IM ? fm : 0][IM ? fn : 0][2 * hh + 1]);
                        }
                    }
                }
            __syncthreads();
            E *Cg = static_cast<E *>(L::kAdd ? a.hout : const_cast<void *>(a.C.p));
            constexpr int ROWS = (CO ? 2 : 1) * MT;
            for (int c = threadIdx.x; c < ROWS * CH; c += NTH) {
                const int r = c / CH, cn = c % CH;
                const int m = r % MT;
                const long long n = n0 + cn * 8;
                if (m < a.M && n < a.Nn) {
                    const long long off = zc + view_off(a.C, m, n) + (r >= MT ? a.C.im : 0);
                    *reinterpret_cast<uint4 *>(Cg + off) =
                        *reinterpret_cast<const uint4 *>(tile + r * BP + cn * 8);
                }
            }
        } else {
#pragma unroll
            for (int fm = 0; fm < FM; fm++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int m = wm * WR + fm * 16 + g + hh * 8;
                    if (m >= a.M) continue;
#pragma unroll
                    for (int fn = 0; fn < FN; fn++) {
                        const long long n = n0 + wn * WC + fn * 8 + 2 * t;
                        if (n >= a.Nn) continue;
                        const long long off = zc + view_off(a.C, m, n);
                        const float v0 = accR[fm][fn][2 * hh], v1 = accR[fm][fn][2 * hh + 1];
                        float2 *c = reinterpret_cast<float2 *>(
                            static_cast<float *>(const_cast<void *>(a.C.p)) + off);
                        if constexpr (EPI == kEpiF32) {
                            *c = make_float2(v0, v1);
                        } else {  // kEpiAccF32
                            float2 o = *c;
                            o.x += a.alpha * v0;
                            o.y += a.alpha * v1;
                            *c = o;
                        }
                    }
                }
        }
        __syncthreads();
        stage = (stage + 1 == ST) ? 0 : stage + 1;
    }
    cp_async_wait<0>();
}

template <int MT, int BN, int WM, int WN, bool AC, bool BC, int EPI, int ST>
inline size_t gemm_sa_smem(int KP)
{
    return SaLayout<MT, BN, WM, AC, BC, EPI, ST>::bytes(KP);
}

// ------------------------------------------------------------ gemm_nt ---
template <typename E, int MT, int NT, int WM, int WN>
__global__ void __launch_bounds__(WM *WN * 32) gemm_nt_kernel(const NtArgs a)
{
    constexpr int NTH = WM * WN * 32, BK = 32, P = BK + 8;
    constexpr int WR = MT / WM, WC = NT / WN;
    constexpr int FM = WR / 16, FN = WC / 8;
    static_assert(WR % 16 == 0 && WC % 16 == 0, "warp tile");
    __shared__ __align__(16) E sA[2][MT * P];
    __shared__ __align__(16) E sB[2][NT * P];

    const long long nchunks = (a.K + a.KC - 1) / a.KC;
    const long long total = nchunks * a.nz;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wm = warp / WN, wn = warp % WN;
    const int g = lane >> 2, t = lane & 3;

    for (long long item = blockIdx.x; item < total; item += gridDim.x) {
        const long long z = item / nchunks;
        const long long k0 = (item % nchunks) * a.KC;
        const long long k1 = min(k0 + a.KC, a.K);
        const long long zA = zoff(z, a.nz2, a.a_z1, a.a_z2);
        const long long zB = zoff(z, a.nz2, a.b_z1, a.b_z2);
        auto issue = [&](long long kt, int st) {
            for (int c = threadIdx.x; c < (MT + NT) * (BK / 8); c += NTH) {
                const int row = c / (BK / 8), ck = c % (BK / 8);
                const long long k = kt + ck * 8;
                if (row < MT) {
                    const bool ok = row < a.M && k < k1;
                    const unsigned kq = fastdiv((unsigned)k, a.awm, a.aws);
                    const long long off =
                        ok ? zA + row * a.a_m + (long long)kq * a.a_blk +
                                 (long long)((unsigned)k - kq * (unsigned)a.a_w)
                           : 0;
                    cp_async16(&sA[st][row * P + ck * 8], static_cast<const E *>(a.A) + off, ok);
                } else {
                    const int n = row - MT;
                    const bool ok = n < a.N && k < k1;
                    const unsigned kq = fastdiv((unsigned)k, a.bwm, a.bws);
                    const long long off =
                        ok ? zB + n * a.b_n + (long long)kq * a.b_blk +
                                 (long long)((unsigned)k - kq * (unsigned)a.b_w)
                           : 0;
                    cp_async16(&sB[st][n * P + ck * 8], static_cast<const E *>(a.B) + off, ok);
                }
            }
        };
        float acc[FM][FN][4];
#pragma unroll
        for (int i = 0; i < FM; i++)
#pragma unroll
            for (int j = 0; j < FN; j++)
#pragma unroll
                for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
        int st = 0;
        issue(k0, 0);
        cp_async_commit();
        for (long long kt = k0; kt < k1; kt += BK, st ^= 1) {
            if (kt + BK < k1) issue(kt + BK, st ^ 1);
            cp_async_commit();
            cp_async_wait<1>();
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; kk += 16) {
                uint32_t af[FM][4];
#pragma unroll
                for (int fm = 0; fm < FM; fm++)
                    ldsm_x4(af[fm], &sA[st][(wm * WR + fm * 16 + (lane & 15)) * P + kk +
                                            (lane >> 4) * 8]);
#pragma unroll
                for (int f2 = 0; f2 < FN / 2; f2++) {
                    uint32_t bq[4];
                    const int nrow = wn * WC + f2 * 16 + (lane & 7) + (lane >> 4) * 8;
                    ldsm_x4(bq, &sB[st][nrow * P + kk + ((lane >> 3) & 1) * 8]);
#pragma unroll
                    for (int fm = 0; fm < FM; fm++) {
                        mma16816<E>(acc[fm][2 * f2], af[fm], bq[0], bq[1]);
                        mma16816<E>(acc[fm][2 * f2 + 1], af[fm], bq[2], bq[3]);
                    }
                }
            }
            __syncthreads();
        }
        cp_async_wait<0>();
        const long long cb = a.c_tab ? (long long)a.c_tab[z] * a.c_tabs : 0;
#pragma unroll
        for (int fm = 0; fm < FM; fm++)
#pragma unroll
            for (int fn = 0; fn < FN; fn++)
#pragma unroll
                for (int r = 0; r < 4; r++) {
                    const int m = wm * WR + fm * 16 + g + (r >> 1) * 8;
                    const int n = wn * WC + fn * 8 + 2 * t + (r & 1);
                    if (m < a.M && n < a.N)
                        atomicAdd(a.C + cb + m * a.c_m + n, a.alpha * acc[fm][fn][r]);
                }
    }
}

}  // namespace fno
}  // namespace sbte
