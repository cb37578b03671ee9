// weights.cu -- FP64 device quadrature of the isotropic convolution weights
// (generate_conv_weights_iso and gHat3, weights.c:181-281):
//
//   W[zeta][xi] = wt(xi) * dfac * prefactor *
//                 int_0^{L_v} r^{lambda+2} [sinc(r a0) sinc(r a2) - sinc(r a1)] dr
//   a0 = mu |zeta|,  a1 = |xi|,  a2 = |xi - mu zeta|.
//
// The reference integrates with adaptive Gauss-Kronrod to 1e-8
// (gsl_integration_qag, weights.c:203).  Here the integral splits into its
// gain and loss parts.  Each part uses composite 16-point Gauss-Legendre
// with panels of at most 6 radians of the highest frequency, which converges
// to round-off.
//  * The loss integral depends on xi alone, so one pass tabulates it for
//    the N^3 columns.
//  * The gain integral is done per row.  A CTA owns one zeta row and puts
//    the row-constant factor w_q r^{lambda+2} sinc(r a0) / r of every node
//    in shared memory.  With the angle-addition split of each node into
//    panel start plus offset, an entry costs (panels + 16) sincos calls.
// One grid covers all rows.  It replaces the reference's OpenMP loop over
// rows (weights.c:269) and the MPI row partition of the stand-alone
// generator (MPIcollisionRoutines.c:252-262).
#include "common.cuh"
#include "kernels.h"

namespace sbte {
namespace {

constexpr int kGL = 16;
constexpr int kMaxNodes = 16 * kWeightMaxPanels;

__device__ __forceinline__ double wtn(int i, int N)
{
    return (i == 0 || i == N - 1) ? 0.5 : 1.0;
}

__device__ __forceinline__ int panels_for(double omega, double L)
{
    int K = (int)ceil(omega * L / 6.0);
    return K < 4 ? 4 : K;
}

// loss[xi] = int_0^{L_v} r^{lambda+2} sinc(r |xi|) dr
__global__ void loss_kernel(double *__restrict__ loss,
                            const double *__restrict__ zeta, WeightParams wp,
                            const double *__restrict__ glx,
                            const double *__restrict__ glw, double a1max)
{
    const int N = wp.N;
    const long long n3 = (long long)N * N * N;
    const int K = panels_for(a1max, wp.L_v);
    const double h = wp.L_v / K;
    for (long long xi = (long long)blockIdx.x * blockDim.x + threadIdx.x; xi < n3;
         xi += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(xi / (N * N)), m = (int)((xi / N) % N), n = (int)(xi % N);
        const double k1 = zeta[l], k2 = zeta[m], k3 = zeta[n];
        const double a1 = sqrt(k1 * k1 + k2 * k2 + k3 * k3);
        double total = 0.0;
        for (int p = 0; p < K; p++) {
            const double mid = (p + 0.5) * h;
            double part = 0.0;
            for (int q = 0; q < kGL; q++) {
                const double r = mid + 0.5 * h * glx[q];
                const double s = (a1 != 0.0) ? sin(r * a1) / (r * a1) : 1.0;
                part += glw[q] * pow(r, wp.lambda + 2) * s;
            }
            total += 0.5 * h * part;
        }
        loss[xi] = total;
    }
}

__global__ void __launch_bounds__(256)
rows_kernel(double *__restrict__ W, int row0, const double *__restrict__ zeta,
            WeightParams wp, const double *__restrict__ glx,
            const double *__restrict__ glw, const double *__restrict__ loss,
            double a2max_extra)
{
    // Node r_pq = s_p + h u_q with panel start s_p = p h and u_q the
    // 16-point rule mapped to (0, 1).  For each entry
    //   sin(a2 r_pq) = sin(a2 s_p) cos(a2 h u_q) + cos(a2 s_p) sin(a2 h u_q),
    // so an entry costs 16 + K sincos evaluations and two length-16 dot
    // products per panel, instead of one sine per node.
    __shared__ double sc[kMaxNodes];  // sc[p*16+q] = row factor of node (p,q)
    __shared__ double sr[kMaxNodes];  // r_pq (for the a2 == 0 entries)
    const int N = wp.N;
    const long long n3 = (long long)N * N * N;
    const long long row = row0 + blockIdx.x;
    const int i = (int)(row / (N * N)), j = (int)((row / N) % N), k = (int)(row % N);
    const double z1 = zeta[i], z2 = zeta[j], z3 = zeta[k];
    const double mu = wp.mu;
    const double a0 = mu * sqrt(z1 * z1 + z2 * z2 + z3 * z3);
    // highest frequency of sinc(r a0) sinc(r a2) over the row
    const double omega = a0 + (a2max_extra + a0);
    int K = panels_for(omega, wp.L_v);
    if (K * kGL > kMaxNodes) K = kMaxNodes / kGL;
    const int P = K * kGL;
    const double h = wp.L_v / K;
    for (int t = threadIdx.x; t < P; t += blockDim.x) {
        const int p = t / kGL, q = t % kGL;
        const double r = (p + 0.5) * h + 0.5 * h * glx[q];
        const double s0 = (a0 != 0.0) ? sin(r * a0) / (r * a0) : 1.0;
        sr[t] = r;
        // 0.5*h*w_q * r^(lambda+2) * sinc(r a0) / r ; the 1/a2 of sinc(r a2)
        // is applied per entry
        sc[t] = 0.5 * h * glw[q] * pow(r, wp.lambda + 2) * s0 / r;
    }
    __syncthreads();
    const double scale = wp.dfac * wp.prefactor;
    double *Wrow = W + (long long)blockIdx.x * n3;
    for (long long xi = threadIdx.x; xi < n3; xi += blockDim.x) {
        const int l = (int)(xi / (N * N)), m = (int)((xi / N) % N), n = (int)(xi % N);
        const double k1 = zeta[l], k2 = zeta[m], k3 = zeta[n];
        const double d1 = k1 - mu * z1, d2 = k2 - mu * z2, d3 = k3 - mu * z3;
        const double a2 = sqrt(d1 * d1 + d2 * d2 + d3 * d3);
        double gain = 0.0;
        if (a2 != 0.0) {
            double cq[kGL], sq[kGL];
#pragma unroll
            for (int q = 0; q < kGL; q++) sincos(a2 * (0.5 * h * (1.0 + glx[q])), &sq[q], &cq[q]);
            for (int p = 0; p < K; p++) {
                double sp, cp;
                sincos(a2 * (p * h), &sp, &cp);
                double dc = 0.0, ds = 0.0;
#pragma unroll
                for (int q = 0; q < kGL; q++) {
                    const double c = sc[p * kGL + q];
                    dc = fma(c, cq[q], dc);
                    ds = fma(c, sq[q], ds);
                }
                gain = fma(sp, dc, gain);
                gain = fma(cp, ds, gain);
            }
            gain /= a2;
        } else {
            for (int t = 0; t < P; t++) gain += sc[t] * sr[t];
        }
        Wrow[xi] = wtn(l, N) * wtn(m, N) * wtn(n, N) * scale * (gain - loss[xi]);
    }
}

// Landau weights (gHat3L, aniso_weights.c:370-400, as generate_conv_weights_AnIso
// fills them, :402-425): one thread per (zeta, xi) entry,
//   W = 2 pi  GL64_{r in [0, L_v]} r^{lambda+2}  GL64_{theta in [0, pi]}
//         sin(th) J0(r xi_perp sin th) (-r^2 |zeta|^2 sin^2 th cos(r a cos th)
//                                       + 4 r |zeta| sin(r a cos th) cos th),
// a = xi.zeta/|zeta|, xi_perp = |xi - a zeta/|zeta||, with the reference's
// 64-point Gauss-Legendre rule (gsl_integration_glfixed) on both axes and its
// operation order.  No trapezoid weights and no prefactor, as in the reference.
__global__ void __launch_bounds__(256)
landau_kernel(double *__restrict__ W, int row0, int nrows, const double *__restrict__ zeta,
              int N, double L_v, double lambda, const double *__restrict__ glx,
              const double *__restrict__ glw)
{
    __shared__ double sx[64], sw[64];
    for (int q = threadIdx.x; q < 64; q += blockDim.x) {
        sx[q] = glx[q];
        sw[q] = glw[q];
    }
    __syncthreads();
    const long long n3 = (long long)N * N * N;
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)nrows * n3) return;
    const long long z = row0 + e / n3, x = e % n3;
    const int k = (int)(z % N), j = (int)((z / N) % N), i = (int)(z / ((long long)N * N));
    const int n = (int)(x % N), m = (int)((x / N) % N), l = (int)(x / ((long long)N * N));
    const double z1 = zeta[i], z2 = zeta[j], z3 = zeta[k];
    const double x1 = zeta[l], x2 = zeta[m], x3 = zeta[n];
    const double zetalen2 = z3 * z3 + z2 * z2 + z1 * z1;
    const double xilen2 = x1 * x1 + x2 * x2 + x3 * x3;
    const double xizeta = x1 * z1 + x2 * z2 + x3 * z3;
    const double zetalen = sqrt(zetalen2);
    double xiperp;
    if (((xilen2 - xizeta * xizeta / zetalen2) < 0) || (zetalen2 == 0))
        xiperp = 0;
    else
        xiperp = sqrt(xilen2 - xizeta * xizeta / zetalen2);
    const double a0 = xiperp, a1 = zetalen2, a2 = zetalen != 0 ? xizeta / zetalen : 0.0,
                 a3 = zetalen;
    const double rmid = 0.5 * L_v, rhalf = 0.5 * L_v;
    const double tmid = 0.5 * M_PI, thalf = 0.5 * M_PI;
    double outer = 0.0;
    for (int p = 0; p < 64; p++) {
        const double r = rmid + rhalf * sx[p];
        double inner = 0.0;
        for (int q = 0; q < 64; q++) {
            const double th = tmid + thalf * sx[q];
            const double st = sin(th), ct = cos(th);
            const double f = st * j0(r * a0 * st) *
                             (-r * r * a1 * st * st * cos(r * a2 * ct) +
                              4 * r * a3 * sin(r * a2 * ct) * ct);
            inner += sw[q] * f;
        }
        outer += sw[p] * (pow(r, lambda + 2) * (thalf * inner));
    }
    W[e] = 2.0 * M_PI * (rhalf * outer);
}

}  // namespace

cudaError_t weights_landau(double *W, int row0, int nrows, const double *zeta, int N,
                           double L_v, double lambda, const double *glx, const double *glw,
                           cudaStream_t st)
{
    const long long total = (long long)nrows * N * N * N;
    if (total <= 0) return cudaSuccess;
    landau_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(W, row0, nrows, zeta, N, L_v,
                                                                   lambda, glx, glw);
    return cudaGetLastError();
}

int weights_panels_needed(const WeightParams &wp)
{
    const double a1max = sqrt(3.0) * wp.zmax;
    const double a0max = wp.mu * a1max;
    const double omega = a0max + (a1max + a0max);
    int K = (int)ceil(omega * wp.L_v / 6.0);
    return K < 4 ? 4 : K;
}

cudaError_t weights_iso(double *W, int row0, int nrows, const double *zeta,
                        const WeightParams &wp, const double *glx,
                        const double *glw, double *loss_scratch,
                        cudaStream_t st)
{
    if (nrows <= 0) return cudaSuccess;
    if (weights_panels_needed(wp) > kWeightMaxPanels) return cudaErrorInvalidValue;
    // |xi| <= sqrt(3) max|zeta_a|; |xi - mu zeta| <= |xi| + mu |zeta|, and
    // the row kernel adds its own a0 = mu |zeta| to that bound.
    const double a1max = sqrt(3.0) * wp.zmax;
    const long long n3 = (long long)wp.N * wp.N * wp.N;
    long long blocks = (n3 + 255) / 256;
    if (blocks > 152 * 8) blocks = 152 * 8;
    loss_kernel<<<(unsigned)blocks, 256, 0, st>>>(loss_scratch, zeta, wp, glx,
                                                  glw, a1max);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    rows_kernel<<<nrows, 256, 0, st>>>(W, row0, zeta, wp, glx, glw, loss_scratch,
                                       a1max);
    return cudaGetLastError();
}

}  // namespace sbte
