// conserve.cu -- FP64 device kernels for the conservation projection
// (conserve.c:207-264), the moments and Maxwellian split of
// find_maxwellians (collisions.c:91-106, momentRoutines.c:58-183), and the
// Euler/RK2 updates of the time loop (boltz.c:206-241).
#include "common.cuh"
#include "kernels.h"

namespace sbte {
namespace {

constexpr int kThreads = 256;
// largest grid side of the separable conservation kernel (its per-axis tables)
constexpr int kConsMaxN = 128;

__device__ __forceinline__ double wt(int i, int N)
{
    // trapezoid weights, collisions.c:48-54
    return (i == 0 || i == N - 1) ? 0.5 : 1.0;
}

// Block-wide sum of K doubles; result valid in every thread.
template <int K>
__device__ void block_sum(double (&x)[K], double *red /* >= 32*K */)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; k++) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x[k] += __shfl_xor_sync(0xffffffffu, x[k], o);
    }
    if (lane == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) red[warp * K + k] = x[k];
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; k++) {
        double s = 0.0;
        for (int w = 0; w < nw; w++) s += red[w * K + k];
        x[k] = s;
    }
    __syncthreads();
}

// solveWithCCt (conserve.c:173-202), one thread.
__device__ void solve_cct(const ConsParams &cp, double *b)
{
    const int n = cp.Ns + 4;
    for (int k = 0; k < n - 1; k++) {
        const int i = cp.pivot[k];
        if (i != k) {
            const double t = b[i];
            b[i] = b[k];
            b[k] = t;
        }
        for (int r = k + 1; r < n; r++) b[r] -= cp.CCt[r][k] * b[k];
    }
    b[n - 1] = b[n - 1] / cp.CCt[n - 1][n - 1];
    for (int i = n - 2; i >= 0; i--) {
        double sum = 0.0;
        for (int j = i + 1; j < n; j++) sum += cp.CCt[i][j] * b[j];
        b[i] = 1.0 / cp.CCt[i][i] * (b[i] - sum);
    }
}

// One species, one CTA per instance.  Grid point (i, j, k) carries the
// prefactor c wt_i wt_j wt_k (c = dv^3 mass, the trapezoid weights of
// conserve.c:207-264), and the moment weights 1, v_i, v_j, v_k, |v|^2 / 2 are
// separable.  So each thread takes (i, k) columns and runs down j against
// the per-j tables e0_j = wt_j, e1_j = wt_j v_j, e2_j = wt_j v_j^2:
//   T0 = sum_j e0_j q,  T1 = sum_j e1_j q,  T2 = sum_j e2_j q,
// then folds the column into the moments with s = c wt_i wt_k:
//   m0 += s T0,  m_x += s v_i T0,  m_y += s T1,  m_z += s v_k T0,
//   m_e += s ((v_i^2 + v_k^2) T0 + T2) / 2.
// The correction prefact (l0 + l1 v_i + l2 v_j + l3 v_k + l4 |v|^2 / 2) is
// s (a e0_j + h_j) with a = l0 + l1 v_i + l3 v_k + l4 (v_i^2 + v_k^2) / 2 and
// h_j = wt_j (l2 v_j + l4 v_j^2 / 2).  That is five FP64 operations per grid
// point, where the direct form spends about forty; FP64 runs at 1/64 of the
// FP32 rate on this GPU, so the count sets the time.  Columns of one i are
// adjacent in k, so each step of j reads contiguous runs of N doubles.
__global__ void __launch_bounds__(kThreads)
conserve_batch_kernel(double *__restrict__ Q, const double *__restrict__ v,
                      ConsParams cp, unsigned int *__restrict__ status)
{
    __shared__ double red[32 * 5];
    __shared__ double lam[8];
    __shared__ double e0[kConsMaxN], e1[kConsMaxN], e2[kConsMaxN], hj[kConsMaxN];
    const int N = cp.N;
    const int NN = N * N;
    double *Qb = Q + (long long)blockIdx.x * NN * N;
    const double c = cp.dv * cp.dv * cp.dv * cp.mass[0];
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double w = wt(j, N), vj = v[j];
        e0[j] = w;
        e1[j] = w * vj;
        e2[j] = w * vj * vj;
    }
    __syncthreads();
    double m[5] = {0, 0, 0, 0, 0};
    for (int p = threadIdx.x; p < NN; p += blockDim.x) {
        const int i = p / N, k = p - (p / N) * N;
        const double *col = Qb + (long long)i * NN + k;
        double t0 = 0.0, t1 = 0.0, t2 = 0.0;
#pragma unroll 8
        for (int j = 0; j < N; j++) {
            const double q = col[(long long)j * N];
            t0 = fma(e0[j], q, t0);
            t1 = fma(e1[j], q, t1);
            t2 = fma(e2[j], q, t2);
        }
        const double vi = v[i], vk = v[k];
        const double s = c * wt(i, N) * wt(k, N);
        const double st0 = s * t0;
        m[0] += st0;
        m[1] = fma(vi, st0, m[1]);
        m[2] = fma(s, t1, m[2]);
        m[3] = fma(vk, st0, m[3]);
        m[4] = fma(0.5 * s, fma(vi * vi + vk * vk, t0, t2), m[4]);
    }
    block_sum<5>(m, red);
    if (threadIdx.x == 0) {
        double b[8];
        for (int t = 0; t < 5; t++) b[t] = m[t];
        solve_cct(cp, b);
        bool finite = true;
        for (int t = 0; t < 5; t++) {
            lam[t] = b[t];
            finite = finite && isfinite(m[t]) && isfinite(b[t]);
        }
        // A NaN or infinity anywhere in Q reaches its moment sums.
        if (!finite && status) atomicOr(status, kStatusNonFinite);
    }
    __syncthreads();
    const double l0 = lam[0], l1 = lam[1], l2 = lam[2], l3 = lam[3], l4 = lam[4];
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        const double vj = v[j];
        hj[j] = wt(j, N) * fma(0.5 * l4, vj * vj, l2 * vj);
    }
    __syncthreads();
    for (int p = threadIdx.x; p < NN; p += blockDim.x) {
        const int i = p / N, k = p - (p / N) * N;
        const double vi = v[i], vk = v[k];
        const double s = c * wt(i, N) * wt(k, N);
        const double a = fma(0.5 * l4, vi * vi + vk * vk, fma(l1, vi, fma(l3, vk, l0)));
        double *col = Qb + (long long)i * NN + k;
#pragma unroll 8
        for (int j = 0; j < N; j++) {
            const double t = fma(a, e0[j], hj[j]);
            col[(long long)j * N] = fma(-s, t, col[(long long)j * N]);
        }
    }
}

// Ns species (Ns <= 4), a single instance; Qp[n*Ns+m] are N^3 arrays.
__global__ void __launch_bounds__(kThreads)
conserve_species_kernel(double **__restrict__ Qp, const double *__restrict__ v,
                        ConsParams cp, unsigned int *__restrict__ status)
{
    __shared__ double red[32 * 8];
    __shared__ double lam[8];
    const int N = cp.N, Ns = cp.Ns;
    const long long n3 = (long long)N * N * N;
    const double dv = cp.dv;
    double m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        for (int s = 0; s < Ns; s++) {
            const double prefact = wt(i, N) * wt(j, N) * wt(k, N) * dv * dv * dv * cp.mass[s];
            const double tm = prefact, tx = prefact * v[i], ty = prefact * v[j],
                         tz = prefact * v[k],
                         te = prefact * 0.5 * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
            for (int n = 0; n < Ns; n++) {
                const double q = Qp[n * Ns + s][x];
                m[s] += q * tm;
                m[Ns] += q * tx;
                m[Ns + 1] += q * ty;
                m[Ns + 2] += q * tz;
                m[Ns + 3] += q * te;
            }
        }
    }
    block_sum<8>(m, red);
    if (threadIdx.x == 0) {
        double b[8];
        for (int t = 0; t < 8; t++) b[t] = m[t];
        solve_cct(cp, b);
        bool finite = true;
        for (int t = 0; t < 8; t++) {
            lam[t] = b[t];
            if (t < Ns + 4) finite = finite && isfinite(m[t]) && isfinite(b[t]);
        }
        if (!finite && status) atomicOr(status, kStatusNonFinite);
    }
    __syncthreads();
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        for (int s = 0; s < Ns; s++) {
            const double prefact = wt(i, N) * wt(j, N) * wt(k, N) * dv * dv * dv * cp.mass[s] / Ns;
            const double tm = prefact, tx = prefact * v[i], ty = prefact * v[j],
                         tz = prefact * v[k],
                         te = prefact * 0.5 * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
            const double d = tm * lam[s] + tx * lam[Ns] + ty * lam[Ns + 1] +
                             tz * lam[Ns + 2] + te * lam[Ns + 3];
            for (int n = 0; n < Ns; n++) Qp[n * Ns + s][x] -= d;
        }
    }
}

// Moments (rho, u, T) of momentRoutines.c and the Maxwellian split of
// find_maxwellians; one CTA per instance.
__global__ void __launch_bounds__(kThreads)
maxwellian_kernel(const double *__restrict__ f, double *__restrict__ M,
                  double *__restrict__ g, const double *__restrict__ Mref,
                  int N, const double *__restrict__ v, double mass, double KB,
                  double *__restrict__ mom, unsigned int *__restrict__ status)
{
    __shared__ double red[32 * 4];
    const long long n3 = (long long)N * N * N;
    const long long off = (long long)blockIdx.x * n3;
    const double dv = v[1] - v[0];
    const double dv3 = dv * dv * dv;
    // density and first moments (getDensity, getBulkVelocity)
    double s[4] = {0, 0, 0, 0};
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        const double w = dv3 * wt(i, N) * wt(j, N) * wt(k, N);
        const double fx = f[off + x];
        s[0] += w * fx;
        s[1] += v[i] * w * fx;
        s[2] += v[j] * w * fx;
        s[3] += v[k] * w * fx;
    }
    block_sum<4>(s, red);
    const double rho = mass * s[0];
    const double u0 = mass * (s[1] / rho), u1 = mass * (s[2] / rho),
                 u2 = mass * (s[3] / rho);
    // temperature (getTemperature)
    double tt[1] = {0};
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        const double t = (v[i] - u0) * (v[i] - u0) + (v[j] - u1) * (v[j] - u1) +
                         (v[k] - u2) * (v[k] - u2);
        tt[0] += t * dv3 * wt(i, N) * wt(j, N) * wt(k, N) * f[off + x];
    }
    block_sum<1>(tt, red);
    const double T = (mass * mass / KB) * (tt[0] / (3.0 * rho));
    const double pre = rho * pow(0.5 / (M_PI * T), 1.5);
    if (threadIdx.x == 0 && status &&
        !(isfinite(rho) && isfinite(u0) && isfinite(u1) && isfinite(u2) && isfinite(T)))
        atomicOr(status, kStatusNonFinite);
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        const double Mx = pre * exp(-(0.5 / T) * ((v[i] - u0) * (v[i] - u0) +
                                                 (v[j] - u1) * (v[j] - u1) +
                                                 (v[k] - u2) * (v[k] - u2)));
        M[off + x] = Mx;
        if (g) g[off + x] = f[off + x] - (Mref ? Mref[off + x] : Mx);
    }
    if (mom && threadIdx.x == 0) {
        mom[5 * blockIdx.x + 0] = rho;
        mom[5 * blockIdx.x + 1] = u0;
        mom[5 * blockIdx.x + 2] = u1;
        mom[5 * blockIdx.x + 3] = u2;
        mom[5 * blockIdx.x + 4] = T;
    }
}

// The per-instance moments that write_streams / write_streams_inhom print
// (output.c:156-213,295-404): getDensity, getBulkVelocity, getTemperature
// (momentRoutines.c:58-69,116-141,168-185), getPressure = rho T (:187-190)
// and getEnergy's positive and negative parts (:146-165).  out[8 b + ...] =
// {rho, u_x, u_y, u_z, T, rho T, E+, E-}.  One CTA per instance, FP64.
__global__ void __launch_bounds__(kThreads)
moments_kernel(const double *__restrict__ f, int N, const double *__restrict__ v, double mass,
               double KB, double *__restrict__ out, unsigned int *__restrict__ status)
{
    __shared__ double red[32 * 4];
    const long long n3 = (long long)N * N * N;
    const double *fb = f + (long long)blockIdx.x * n3;
    const double dv = v[1] - v[0];
    const double dv3 = dv * dv * dv;
    double s[4] = {0, 0, 0, 0};
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        const double w = dv3 * wt(i, N) * wt(j, N) * wt(k, N);
        const double fx = fb[x];
        s[0] += w * fx;
        s[1] += v[i] * w * fx;
        s[2] += v[j] * w * fx;
        s[3] += v[k] * w * fx;
    }
    block_sum<4>(s, red);
    const double rho = mass * s[0];
    const double u0 = mass * (s[1] / rho), u1 = mass * (s[2] / rho), u2 = mass * (s[3] / rho);
    double t[3] = {0, 0, 0};
    for (int x = threadIdx.x; x < (int)n3; x += blockDim.x) {
        const int i = x / (N * N), j = (x / N) % N, k = x % N;
        const double w = dv3 * wt(i, N) * wt(j, N) * wt(k, N);
        const double fx = fb[x];
        t[0] += ((v[i] - u0) * (v[i] - u0) + (v[j] - u1) * (v[j] - u1) +
                 (v[k] - u2) * (v[k] - u2)) * w * fx;
        const double e = w * fx * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
        if (e > 0) t[1] += e; else t[2] -= e;
    }
    block_sum<3>(t, red);
    if (threadIdx.x == 0) {
        const double T = (mass * mass / KB) * (t[0] / (3.0 * rho));
        double *o = out + 8 * (long long)blockIdx.x;
        o[0] = rho; o[1] = u0; o[2] = u1; o[3] = u2; o[4] = T; o[5] = rho * T;
        o[6] = t[1]; o[7] = t[2];
        bool finite = true;
        for (int q = 0; q < 8; q++) finite = finite && isfinite(o[q]);
        if (!finite && status) atomicOr(status, kStatusNonFinite);
    }
}

__global__ void axpy_kernel(double *__restrict__ y, const double *__restrict__ x,
                            const double *__restrict__ q, double a_y, double a_x,
                            double a_q, long long n)
{
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        double r = (a_y != 0.0) ? a_y * y[t] : 0.0;  // y is not read when a_y == 0
        if (x) r += a_x * x[t];
        if (q) r += a_q * q[t];
        y[t] = r;
    }
}

}  // namespace

cudaError_t conserve_batch(double *Q, int B, const double *v,
                           const ConsParams &cp, cudaStream_t st, unsigned int *status)
{
    if (B < 1) return cudaSuccess;
    if (cp.N < 2 || cp.N > kConsMaxN) return cudaErrorInvalidValue;
    conserve_batch_kernel<<<B, kThreads, 0, st>>>(Q, v, cp, status);
    return cudaGetLastError();
}

cudaError_t conserve_species(double **Qptrs_dev, const double *v,
                             const ConsParams &cp, cudaStream_t st, unsigned int *status)
{
    conserve_species_kernel<<<1, kThreads, 0, st>>>(Qptrs_dev, v, cp, status);
    return cudaGetLastError();
}

cudaError_t maxwellian_split(const double *f, double *M, double *g,
                             const double *Mref, int B, int N, const double *v,
                             double mass, double KB, double *moments_out,
                             cudaStream_t st, unsigned int *status)
{
    if (B < 1) return cudaSuccess;
    maxwellian_kernel<<<B, kThreads, 0, st>>>(f, M, g, Mref, N, v, mass, KB,
                                              moments_out, status);
    return cudaGetLastError();
}

cudaError_t moments_batch(const double *f, int B, int N, const double *v, double mass,
                          double KB, double *out, cudaStream_t st, unsigned int *status)
{
    if (B < 1) return cudaSuccess;
    moments_kernel<<<B, kThreads, 0, st>>>(f, N, v, mass, KB, out, status);
    return cudaGetLastError();
}

cudaError_t axpy_update(double *y, const double *x, const double *q, double a_y,
                        double a_x, double a_q, long long n, cudaStream_t st)
{
    if (n <= 0) return cudaSuccess;
    long long blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    axpy_kernel<<<(unsigned)blocks, 256, 0, st>>>(y, x, q, a_y, a_x, a_q, n);
    return cudaGetLastError();
}

}  // namespace sbte
