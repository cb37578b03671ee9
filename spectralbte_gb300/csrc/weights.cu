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

// ---------------------------------------------------- closed-form weights ---
// The radial integral of ghat (weights.c:156-160) in closed form for
// lambda = 0 and 1, derived from the integrand.  With s(x) = sin x / x and
// q(x) = (1 - cos x) / x^2 = s(x/2)^2 / 2:
//   gain, lambda 0: int_0^L r^2 s(ra) s(rb) dr = L/(2ab) [s(Ld) - s(Le)]
//   gain, lambda 1: int_0^L r^3 s(ra) s(rb) dr = L^2/(2ab) [s(Ld) - q(Ld) - s(Le) + q(Le)]
//     (d = a - b, e = a + b: 2 sin A sin B = cos(A - B) - cos(A + B), and
//     int_0^L r cos(rk) dr = L^2 [s(Lk) - q(Lk)]);
//   loss, lambda 0: int_0^L r^2 s(rc) dr = (sin x - x cos x) / c^3
//   loss, lambda 1: int_0^L r^3 s(rc) dr = ((2 - x^2) cos x + 2 x sin x - 2) / c^4
//     (x = Lc; below x = 1/2 the series L^(lambda+3) sum_k (-1)^k x^2k /
//     ((2k+1)! (2k+lambda+3)) avoids the cancellation).
// A gain argument of exactly 0 turns the gain into the loss form of the
// other.  The host admits a grid only when every nonzero gain argument is at
// least 1/2 / L (otherwise 1/(ab) would cost digits).
__device__ __forceinline__ double sinc_d(double x) { return x != 0.0 ? sin(x) / x : 1.0; }

__device__ double loss_closed_d(double c, int lam, double L)
{
    const double x = L * c;
    const double Lp = lam == 0 ? L * L * L : L * L * L * L;
    if (x < 0.5) {
        double term = 1.0, sum = 0.0;
        for (int k = 0; k < 12; k++) {
            sum += term / (2.0 * k + lam + 3.0);
            term *= -x * x / ((2.0 * k + 2.0) * (2.0 * k + 3.0));
        }
        return Lp * sum;
    }
    double sx, cx;
    sincos(x, &sx, &cx);
    if (lam == 0) return (sx - x * cx) / (c * c * c);
    return ((2.0 - x * x) * cx + 2.0 * x * sx - 2.0) / (c * c * c * c);
}

__device__ __forceinline__ double q_stable_d(double x)
{
    const double h = sinc_d(0.5 * x);
    return 0.5 * h * h;
}

__device__ double ghat_closed_d(double a0, double a1, double a2, int lam, double L)
{
    double gain;
    if (a0 == 0.0 && a2 == 0.0)
        gain = lam == 0 ? L * L * L / 3.0 : L * L * L * L / 4.0;
    else if (a0 == 0.0)
        gain = loss_closed_d(a2, lam, L);
    else if (a2 == 0.0)
        gain = loss_closed_d(a0, lam, L);
    else {
        const double d = L * (a0 - a2), e = L * (a0 + a2);
        if (lam == 0)
            gain = L / (2.0 * a0 * a2) * (sinc_d(d) - sinc_d(e));
        else
            gain = L * L / (2.0 * a0 * a2) * (sinc_d(d) - q_stable_d(d) - sinc_d(e) + q_stable_d(e));
    }
    return gain - loss_closed_d(a1, lam, L);
}

// W[zeta = (i, j, k)][xi = (l, m, n)] (weights.c:265-281 with the closed
// radial integral): wt(l) wt(m) wt(n) dfac prefactor ghat(a0, a1, a2),
// a0 = mu |zeta|, a1 = |xi|, a2 = |xi - mu zeta|.
__device__ __forceinline__ double w_closed(const double *__restrict__ zeta, const WeightParams &wp,
                                           int lam, int i, int j, int k, int l, int m, int n)
{
    const int N = wp.N;
    const double z1 = zeta[i], z2 = zeta[j], z3 = zeta[k];
    const double k1 = zeta[l], k2 = zeta[m], k3 = zeta[n];
    const double mu = wp.mu;
    const double a0 = mu * sqrt(z1 * z1 + z2 * z2 + z3 * z3);
    const double a1 = sqrt(k1 * k1 + k2 * k2 + k3 * k3);
    const double d1 = k1 - mu * z1, d2 = k2 - mu * z2, d3 = k3 - mu * z3;
    const double a2 = sqrt(d1 * d1 + d2 * d2 + d3 * d3);
    // a zero of exact arithmetic that rounding left as a few ulps: the gain is
    // continuous there, and its a2 -> 0 branch is the accurate one
    return wtn(l, N) * wtn(m, N) * wtn(n, N) * wp.dfac *
           (wp.prefactor * ghat_closed_d(a0 < wp.ztol ? 0.0 : a0, a1, a2 < wp.ztol ? 0.0 : a2,
                                         lam, wp.L_v));
}

// FP64 rows [row0, row0 + nrows) of the table, row-major.
__global__ void __launch_bounds__(256)
iso_closed_kernel(double *__restrict__ W, int row0, int nrows, const double *__restrict__ zeta,
                  WeightParams wp, int lam)
{
    const int N = wp.N;
    const long long n3 = (long long)N * N * N;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < nrows * n3;
         e += (long long)gridDim.x * blockDim.x) {
        const long long z = row0 + e / n3, x = e % n3;
        W[e] = w_closed(zeta, wp, lam, (int)(z / (N * N)), (int)((z / N) % N), (int)(z % N),
                        (int)(x / (N * N)), (int)((x / N) % N), (int)(x % N));
    }
}

// The row-pair FP32 table of the warp-specialised convolution, from the
// closed form, with no FP64 table: for zeta-row (zx, zy) (one CTA) and each
// run slot r (rows whose partner s(r) = (zeta + N/2 - r) mod N does not
// precede them), Wsym[zrow][slot][zz][xz] = W[zeta][r, xz] +
// W[zeta][s(r), (zz + N/2 - xz) mod N] (the second term only when s(r) != r),
// summed in FP64 and rounded once, as weights_to_sym_f32 does from a table.
__global__ void __launch_bounds__(256)
sym_closed_kernel(float *__restrict__ Wsym, const double *__restrict__ zeta, WeightParams wp,
                  int lam)
{
    __shared__ short rows[64 * 64 / 2 + 2];
    __shared__ int nrows;
    const int N = wp.N, nn = N * N, h = N / 2;
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
            w = w_closed(zeta, wp, lam, zx, zy, zz, r / N, r % N, xz);
            if (sx * N + sy != r) {
                const int sz = (zz + h - xz + N) % N;
                w += w_closed(zeta, wp, lam, zx, zy, zz, sx, sy, sz);
            }
        }
        out[t] = (float)w;
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

// gHat3 of the grazing-collision generator (MPIcollisionRoutines.c:33-205)
// for one (zeta, xi) pair per CTA: pairs[6 u .. 6 u + 5] = zeta1..3, xi1..3.
//   W = 4 pi^2 int_0^{L_v} r^{lambda+2} int_0^pi sin(phi) J0(r sin(phi) xp)
//         [I1(r, phi) + C(r, phi) taylor] dphi dr,
//   I1 = int_{sqrt g}^pi (8/pi) g theta^-4 [cos(a7 (1 - cos th) - a6)
//         J0(a8 sin th) - cos a6] dth,
// a6 = r cos(phi) xz, a7 = r cos(phi) zl / 2, a8 = r sin(phi) zl / 2,
// C = -a8^2 cos(a6) / 4 + a7 sin(a6) / 2, taylor = (2/pi) log g / log sin(g/2)
// (the reference's analytic Coulomb-case term for theta < sqrt g).  Every
// level is composite 16-point Gauss-Legendre: npan equal panels in r and phi,
// and the nte panels between the edges te[] in theta (graded geometrically
// from sqrt g, where the integrand grows like theta^-2).  The reference
// integrates with GSL QAG / CQUAD to 1e-6; these rules converge to ~1e-13.
// The threads of a CTA share the npan^2 * 256 (r, phi) nodes; each node's
// theta integral runs in one thread, and a block sum finishes the weight.
__global__ void __launch_bounds__(256)
graze_kernel(double *__restrict__ out, const double *__restrict__ pairs, double L_v,
             double lambda, double glance, double taylor, int npan,
             const double *__restrict__ te, int nte, const double *__restrict__ glx,
             const double *__restrict__ glw)
{
    __shared__ double sx[16], sw[16], se[64], red[8];
    if (threadIdx.x < 16) {
        sx[threadIdx.x] = glx[threadIdx.x];
        sw[threadIdx.x] = glw[threadIdx.x];
    }
    for (int q = threadIdx.x; q <= nte; q += blockDim.x) se[q] = te[q];
    __syncthreads();
    const double *q = pairs + 6LL * blockIdx.x;
    const double z1 = q[0], z2 = q[1], z3 = q[2], x1 = q[3], x2 = q[4], x3 = q[5];
    const double zetalen2 = z1 * z1 + z2 * z2 + z3 * z3;
    const double xilen2 = x1 * x1 + x2 * x2 + x3 * x3;
    const double xizeta = x1 * z1 + x2 * z2 + x3 * z3;
    const double zl = sqrt(zetalen2);
    double xp;
    if (((xilen2 - xizeta * xizeta / zetalen2) < 0) || (zetalen2 == 0))
        xp = 0;
    else
        xp = sqrt(xilen2 - xizeta * xizeta / zetalen2);
    const double xz = zl != 0 ? xizeta / zl : 0.0;
    const double hr = L_v / npan, hp = M_PI / npan;
    const int nn = npan * 16;
    double acc = 0.0;
    for (int t = threadIdx.x; t < nn * nn; t += blockDim.x) {
        const int ir = t / nn, ip = t - ir * nn;
        const double r = hr * (ir >> 4) + 0.5 * hr * (sx[ir & 15] + 1.0);
        const double wr = 0.5 * hr * sw[ir & 15];
        const double phi = hp * (ip >> 4) + 0.5 * hp * (sx[ip & 15] + 1.0);
        const double wp = 0.5 * hp * sw[ip & 15];
        double sph, cph;
        sincos(phi, &sph, &cph);
        const double a6 = r * cph * xz, a7 = 0.5 * r * cph * zl, a8 = 0.5 * r * sph * zl;
        double s6, c6;
        sincos(a6, &s6, &c6);
        double i1 = 0.0;
        for (int pt = 0; pt < nte; pt++) {
            const double t0 = se[pt], ht = se[pt + 1] - se[pt];
            double s = 0.0;
            for (int qt = 0; qt < 16; qt++) {
                const double th = t0 + 0.5 * ht * (sx[qt] + 1.0);
                double sth, cth;
                sincos(th, &sth, &cth);
                const double bcos = (8.0 / M_PI) * (glance / (th * th)) / (th * th);
                s += sw[qt] * bcos * (cos(a7 * (1.0 - cth) - a6) * j0(a8 * sth) - c6);
            }
            i1 += 0.5 * ht * s;
        }
        const double C = -0.25 * a8 * a8 * c6 + 0.5 * a7 * s6;
        acc += wr * pow(r, lambda + 2) * wp * sph * j0(r * sph * xp) * (i1 + C * taylor);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double tot = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[w];
        out[blockIdx.x] = 4.0 * M_PI * M_PI * tot;
    }
}

// W[e] = vals[map[e]] for the n entries of a weight table.
__global__ void scatter_kernel(double *__restrict__ W, const double *__restrict__ vals,
                               const int *__restrict__ map, long long n)
{
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n;
         e += (long long)gridDim.x * blockDim.x)
        W[e] = vals[map[e]];
}

}  // namespace

cudaError_t weights_graze(double *vals, const double *pairs, int npairs, double L_v,
                          double lambda, double glance, int npan, const double *te, int nte,
                          const double *glx, const double *glw, cudaStream_t st)
{
    if (npairs <= 0) return cudaSuccess;
    if (nte < 1 || nte > 62 || npan < 1 || !(glance > 0.0)) return cudaErrorInvalidValue;
    const double taylor = (2.0 / M_PI) * log(glance) / log(sin(0.5 * glance));
    graze_kernel<<<npairs, 256, 0, st>>>(vals, pairs, L_v, lambda, glance, taylor, npan, te,
                                         nte, glx, glw);
    return cudaGetLastError();
}

cudaError_t weights_scatter(double *W, const double *vals, const int *map, long long n,
                            cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    scatter_kernel<<<(unsigned)blocks, 256, 0, st>>>(W, vals, map, n);
    return cudaGetLastError();
}

cudaError_t weights_iso_closed(double *W, int row0, int nrows, const double *zeta,
                               const WeightParams &wp, cudaStream_t st)
{
    const int lam = wp.lambda == 0.0 ? 0 : (wp.lambda == 1.0 ? 1 : -1);
    if (lam < 0) return cudaErrorInvalidValue;
    const long long total = (long long)nrows * wp.N * wp.N * wp.N;
    if (total <= 0) return cudaSuccess;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    iso_closed_kernel<<<(unsigned)blocks, 256, 0, st>>>(W, row0, nrows, zeta, wp, lam);
    return cudaGetLastError();
}

cudaError_t weights_sym_closed(float *Wsym, const double *zeta, const WeightParams &wp,
                               cudaStream_t st)
{
    const int lam = wp.lambda == 0.0 ? 0 : (wp.lambda == 1.0 ? 1 : -1);
    if (lam < 0 || wp.N % 2 != 0 || wp.N < 2 || wp.N > 64) return cudaErrorInvalidValue;
    sym_closed_kernel<<<wp.N * wp.N, 256, 0, st>>>(Wsym, zeta, wp, lam);
    return cudaGetLastError();
}

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
