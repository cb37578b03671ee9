// fno_fused.cuh -- the last inverse axis pass of a spectral layer fused with
// its channel mix, for the N = 32, width 64, 12-mode network.
//
// Unfused, a layer ends with two streaming GEMMs:
//   S[p][d][b]  = Re sum_mk G[k][mk] U2[i][j][mk][d][b]        (p = (i, j, k))
//   h'[p][d][b] = act(sum_c W[d][c] h[p][c][b] + bias[d] + S[p][d][b])
// and S (one activation-sized tensor) goes out to HBM and back.  Here one
// work item is a row (i, j) and BB = 8 consecutive instances: both products
// run from shared memory and S never leaves the CTA.
//   GEMM 1: S[k][(d, b)] = sum_kappa A1[k][kappa] U2[kappa][(d, b)],
//           kappa = (part, mk), A1 = [Gr | -Gi]   (M = 32, K = 24 -> 32, N = 512)
//   GEMM 2: Z[d][(k, b)] = sum_c W[d][c] H[c][(k, b)]         (M = 64, K = 64, N = 256)
// S is rounded to the element type where the unfused path stores it, and the
// layer output overwrites S's tile slot (each element has one owner thread)
// before leaving as 16-byte rows.  When the next layer needs its first
// forward axis pass, a third product runs on that tile as it stands:
//   GEMM 3: T1[kappa][(d, b)] = sum_k [Fr; Fi][kappa][k] h'[k][(d, b)]
// (the layout of T1 is that of U2), so the next layer skips re-reading h'.
// Eight warps, 112 KB of shared memory, two CTAs per SM.
#pragma once

#include "fno_gemm.cuh"

namespace sbte {
namespace fno {

struct FusedArgs {
    const void *U2;      // [i][j][2][mk][d][b]
    const void *H;       // [p][c][b]
    void *Hout;          // [p][d][b]
    float *zst;          // optional FP32 pre-activation, [p][d][b]
    const float *G;      // inverse axis matrix: re [x][m], im at + N * Km
    const float *F;      // forward axis matrix: re [m][x], im at + Km * N
    void *T1;            // optional: the next layer's first forward pass output
    const float *W;      // [d][c]
    const float *bias;   // [d]
    int act;             // 1: GELU
    int Bp;              // instances (multiple of 8)
};

template <typename E, int NN, int C, int KM> struct FusedLayout {
    static constexpr int BB = 8;
    static constexpr int KAP = 2 * KM;                 // GEMM-1 depth
    static constexpr int K1 = (KAP + 15) / 16 * 16;    // padded
    static constexpr int NS = C * BB;                  // S columns (d, b)
    static constexpr int NH = NN * BB;                 // H columns (k, b)
    static constexpr int PG = K1 + 8, PW = C + 8, PU = NS + 8, PH = NH + 8, PS = NS + 8;
    static constexpr int PF = NN + 8;
    static constexpr int oG = 0, oW = oG + NN * PG, oU = oW + C * PW, oH = oU + K1 * PU,
                         oS = oH + C * PH, oF = oS + NN * PS, total = oF + K1 * PF;
    static constexpr size_t bytes = sizeof(E) * (size_t)total;
    static constexpr int NTH = 256;
    static_assert(NN == 32 && C == 64, "the fused layer is written for N = 32, width 64");
    static_assert(NS % (8 * 64) == 0 && NH % (8 * 32) == 0, "warp tiling");
};

template <typename E, int NN, int C, int KM>
__global__ void __launch_bounds__(256) fused_layer_kernel(const FusedArgs a)
{
    using L = FusedLayout<E, NN, C, KM>;
    using T2 = typename Elem<E>::T2;
    constexpr int BB = L::BB, NTH = L::NTH;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    E *sm = reinterpret_cast<E *>(smem_raw);
    E *sG = sm + L::oG, *sW = sm + L::oW, *sU = sm + L::oU, *sH = sm + L::oH, *sS = sm + L::oS;
    E *sF = sm + L::oF;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = lane >> 2, t = lane & 3;
    const long long Bp = a.Bp, CB = (long long)C * Bp;

    // the two small operands, once per CTA
    for (int e = tid; e < NN * L::K1; e += NTH) {
        const int k = e / L::K1, kap = e % L::K1;
        float v = 0.f;
        if (kap < KM) v = a.G[k * KM + kap];
        else if (kap < L::KAP) v = -a.G[NN * KM + k * KM + (kap - KM)];
        sG[k * L::PG + kap] = Elem<E>::cvt(v);
    }
    for (int e = tid; e < C * C; e += NTH) sW[(e / C) * L::PW + e % C] = Elem<E>::cvt(a.W[e]);
    // [Fr; Fi][kappa][k]: kappa < KM real rows, then imaginary rows, then zeros
    for (int e = tid; e < L::K1 * NN; e += NTH) {
        const int kap = e / NN, k = e % NN;
        float v = 0.f;
        if (kap < KM) v = a.F[kap * NN + k];
        else if (kap < L::KAP) v = a.F[KM * NN + (kap - KM) * NN + k];
        sF[kap * L::PF + k] = Elem<E>::cvt(v);
    }
    // rows kappa >= KAP of the U2 tile stay zero
    for (int e = tid; e < (L::K1 - L::KAP) * L::PU; e += NTH) sU[L::KAP * L::PU + e] = Elem<E>::cvt(0.f);

    const unsigned nbc = (unsigned)(Bp / BB);
    const unsigned total = (unsigned)(NN * NN) * nbc;
    const E *U2 = static_cast<const E *>(a.U2);
    const E *Hg = static_cast<const E *>(a.H);
    E *Ho = static_cast<E *>(a.Hout);
    for (unsigned item = blockIdx.x; item < total; item += gridDim.x) {
        const unsigned ij = item / nbc;
        const long long b0 = (long long)(item - ij * nbc) * BB;
        __syncthreads();  // previous item done with sU, sH, sS
        // U2[ij][part][mk][d][b0..b0+8) -> sU[part*KM + mk][d*8 + b]
        for (int c = tid; c < L::KAP * C; c += NTH) {
            const int kap = c / C, d = c % C;
            const long long off = (long long)ij * 2 * KM * CB + (long long)kap * CB + d * Bp + b0;
            cp_async16(sU + kap * L::PU + d * BB, U2 + off, true);
        }
        // H[(ij, k)][c][b0..b0+8) -> sH[c][k*8 + b]
        for (int e = tid; e < NN * C; e += NTH) {
            const int k = e / C, c = e % C;
            const long long off = ((long long)ij * NN + k) * CB + (long long)c * Bp + b0;
            cp_async16(sH + c * L::PH + k * BB, Hg + off, true);
        }
        cp_async_commit();
        cp_async_wait<0>();
        __syncthreads();

        // ---- GEMM 1: S[k][(d,b)], warp w owns columns [64 w, 64 w + 64)
        {
            float acc[2][8][4];
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 8; j++)
#pragma unroll
                    for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
#pragma unroll
            for (int kk = 0; kk < L::K1; kk += 16) {
                uint32_t af[2][4];
#pragma unroll
                for (int fm = 0; fm < 2; fm++)
                    ldsm_x4(af[fm], sG + (fm * 16 + (lane & 15)) * L::PG + kk + (lane >> 4) * 8);
#pragma unroll
                for (int f2 = 0; f2 < 4; f2++) {
                    uint32_t bq[4];
                    ldsm_x4_t(bq, sU + (kk + (lane & 15)) * L::PU + warp * 64 + f2 * 16 +
                                      (lane >> 4) * 8);
#pragma unroll
                    for (int fm = 0; fm < 2; fm++) {
                        mma16816<E>(acc[fm][2 * f2], af[fm], bq[0], bq[1]);
                        mma16816<E>(acc[fm][2 * f2 + 1], af[fm], bq[2], bq[3]);
                    }
                }
            }
#pragma unroll
            for (int fm = 0; fm < 2; fm++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int k = fm * 16 + g + hh * 8;
#pragma unroll
                    for (int fn = 0; fn < 8; fn++) {
                        const int col = warp * 64 + fn * 8 + 2 * t;
                        *reinterpret_cast<T2 *>(sS + k * L::PS + col) =
                            Elem<E>::cvt2(acc[fm][fn][2 * hh], acc[fm][fn][2 * hh + 1]);
                    }
                }
        }
        __syncthreads();

        // ---- GEMM 2: Z[d][(k,b)], warp w owns columns [32 w, 32 w + 32): k = 4 w .. 4 w + 3
        {
            float acc[4][4][4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++)
#pragma unroll
                    for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
#pragma unroll
            for (int kk = 0; kk < C; kk += 16) {
                uint32_t af[4][4];
#pragma unroll
                for (int fm = 0; fm < 4; fm++)
                    ldsm_x4(af[fm], sW + (fm * 16 + (lane & 15)) * L::PW + kk + (lane >> 4) * 8);
#pragma unroll
                for (int f2 = 0; f2 < 2; f2++) {
                    uint32_t bq[4];
                    ldsm_x4_t(bq, sH + (kk + (lane & 15)) * L::PH + warp * 32 + f2 * 16 +
                                      (lane >> 4) * 8);
#pragma unroll
                    for (int fm = 0; fm < 4; fm++) {
                        mma16816<E>(acc[fm][2 * f2], af[fm], bq[0], bq[1]);
                        mma16816<E>(acc[fm][2 * f2 + 1], af[fm], bq[2], bq[3]);
                    }
                }
            }
            // epilogue: z = acc + bias + S, written back over S's slot
#pragma unroll
            for (int fm = 0; fm < 4; fm++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int d = fm * 16 + g + hh * 8;
                    const float bd = a.bias[d];
#pragma unroll
                    for (int fn = 0; fn < 4; fn++) {
                        const int k = warp * 4 + fn, b = 2 * t;  // column (k, b)
                        T2 *slot = reinterpret_cast<T2 *>(sS + k * L::PS + d * BB + b);
                        const float2 sv = Elem<E>::f2(*slot);
                        const float z0 = acc[fm][fn][2 * hh] + bd + sv.x;
                        const float z1 = acc[fm][fn][2 * hh + 1] + bd + sv.y;
                        if (a.zst) {
                            const long long off =
                                ((long long)ij * NN + k) * CB + (long long)d * Bp + b0 + b;
                            *reinterpret_cast<float2 *>(a.zst + off) = make_float2(z0, z1);
                        }
                        if (a.act) {
                            const float2 o = gelu2_f(make_float2(z0, z1));
                            *slot = Elem<E>::cvt2(o.x, o.y);
                        } else {
                            *slot = Elem<E>::cvt2(z0, z1);
                        }
                    }
                }
        }
        __syncthreads();
        // h'[(ij, k)][d][b0..b0+8) from sS[k][d*8 + b]
        for (int e = tid; e < NN * C; e += NTH) {
            const int k = e / C, d = e % C;
            const long long off = ((long long)ij * NN + k) * CB + (long long)d * Bp + b0;
            *reinterpret_cast<uint4 *>(Ho + off) =
                *reinterpret_cast<const uint4 *>(sS + k * L::PS + d * BB);
        }
        if (a.T1) {
            // ---- GEMM 3: T1[kappa][(d,b)] from h' in sS, staged in the U2 slot
            float acc[2][8][4];
#pragma unroll
            for (int i = 0; i < 2; i++)
#pragma unroll
                for (int j = 0; j < 8; j++)
#pragma unroll
                    for (int r = 0; r < 4; r++) acc[i][j][r] = 0.f;
#pragma unroll
            for (int kk = 0; kk < NN; kk += 16) {
                uint32_t af[2][4];
#pragma unroll
                for (int fm = 0; fm < 2; fm++)
                    ldsm_x4(af[fm], sF + (fm * 16 + (lane & 15)) * L::PF + kk + (lane >> 4) * 8);
#pragma unroll
                for (int f2 = 0; f2 < 4; f2++) {
                    uint32_t bq[4];
                    ldsm_x4_t(bq, sS + (kk + (lane & 15)) * L::PS + warp * 64 + f2 * 16 +
                                      (lane >> 4) * 8);
#pragma unroll
                    for (int fm = 0; fm < 2; fm++) {
                        mma16816<E>(acc[fm][2 * f2], af[fm], bq[0], bq[1]);
                        mma16816<E>(acc[fm][2 * f2 + 1], af[fm], bq[2], bq[3]);
                    }
                }
            }
#pragma unroll
            for (int fm = 0; fm < 2; fm++)
#pragma unroll
                for (int hh = 0; hh < 2; hh++) {
                    const int kap = fm * 16 + g + hh * 8;
                    if (kap >= L::KAP) continue;  // rows KAP..K1 of sU stay zero
#pragma unroll
                    for (int fn = 0; fn < 8; fn++) {
                        const int col = warp * 64 + fn * 8 + 2 * t;
                        *reinterpret_cast<T2 *>(sU + kap * L::PU + col) =
                            Elem<E>::cvt2(acc[fm][fn][2 * hh], acc[fm][fn][2 * hh + 1]);
                    }
                }
            __syncthreads();
            E *T1 = static_cast<E *>(a.T1);
            for (int c = tid; c < L::KAP * C; c += NTH) {
                const int kap = c / C, d = c % C;
                const long long off =
                    (long long)ij * 2 * KM * CB + (long long)kap * CB + d * Bp + b0;
                *reinterpret_cast<uint4 *>(T1 + off) =
                    *reinterpret_cast<const uint4 *>(sU + kap * L::PU + d * BB);
            }
        }
    }
}

}  // namespace fno
}  // namespace sbte
