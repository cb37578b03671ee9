// transport.cu -- device transport for the 1D-3V solver: first-order upwind
// (upwindOne, transportroutines.c:94-238), second-order minmod with its
// wall reconstruction (upwindTwo, :241-470), and diffuse-reflection walls
// (setDiffuseReflectionBC, boundaryConditions.c:39-96).  All cells of a
// run stay in one device array [cells][N^3], so the reference's MPI halo
// exchange (transportroutines.c:107-172, 261-344) becomes plain neighbour
// reads.
#include "common.cuh"
#include "kernels.h"

namespace sbte {
namespace {

__device__ __forceinline__ double wtn(int i, int N)
{
    return (i == 0 || i == N - 1) ? 0.5 : 1.0;
}

__device__ __forceinline__ double minmod3(double a, double b, double c)
{
    // transportroutines.c:80-90
    if ((a > 0) && (b > 0) && (c > 0)) return fmin(fmin(a, b), c);
    if ((a < 0) && (b < 0) && (c < 0)) return fmax(fmax(a, b), c);
    return 0.0;
}

// Diffuse reflection: sigmaW from the outgoing half of `in`, then the wall
// Maxwellian on the incoming half of `out` (in == out allowed: the halves
// are disjoint).  One CTA per wall; up to two walls per launch.
struct BcJob {
    const double *in;
    double *out;
    double TW;
    int right;
};

__global__ void __launch_bounds__(256)
diffuse_bc_kernel(BcJob j0, BcJob j1, int njobs, const double *__restrict__ v, int N,
                  double mass, double KB)
{
    __shared__ double red[32];
    const BcJob j = blockIdx.x == 0 ? j0 : j1;
    if ((int)blockIdx.x >= njobs) return;
    const int half = N / 2;
    const int ilo = j.right ? half : 0;
    const long long nh = (long long)half * N * N;
    const double h_v = v[1] - v[0];
    double s = 0.0;
    for (int t = threadIdx.x; t < (int)nh; t += blockDim.x) {
        const int i = ilo + t / (N * N);
        const int jj = (t / N) % N, k = t % N;
        s += v[i] * wtn(i, N) * wtn(jj, N) * wtn(k, N) * h_v * h_v * h_v *
             j.in[k + (long long)N * (jj + (long long)N * i)];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    double sigmaW = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) sigmaW += red[w];
    sigmaW *= (j.right ? 1.0 : -1.0) * sqrt(2.0 * M_PI * mass / (KB * j.TW));
    const double pre = sigmaW * pow(0.5 * mass / (M_PI * KB * j.TW), 1.5);
    const double ex = -0.5 * mass / (KB * j.TW);
    const int olo = j.right ? 0 : half;
    for (int t = threadIdx.x; t < (int)nh; t += blockDim.x) {
        const int i = olo + t / (N * N);
        const int jj = (t / N) % N, k = t % N;
        j.out[k + (long long)N * (jj + (long long)N * i)] =
            pre * exp(ex * (v[i] * v[i] + v[jj] * v[jj] + v[k] * v[k]));
    }
}

// First-order upwind for cells 1..nX (transportroutines.c:203-237).
__global__ void upwind1_kernel(const double *__restrict__ f, double *__restrict__ fc,
                               const double *__restrict__ v, const double *__restrict__ dx,
                               int N, int nX, double dt, int ic)
{
    const long long n3 = (long long)N * N * N;
    const long long total = (long long)nX * n3;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const unsigned tc = (unsigned)t / (unsigned)n3;  // 32-bit: nX N^3 < 2^31
        const int l = 1 + (int)tc;
        const long long q = (long long)((unsigned)t - tc * (unsigned)n3);
        const int i = (int)q / (N * N), j = ((int)q / N) % N;
        const double *fl = f + (long long)l * n3;
        const double CFL = dt * v[i] / dx[l];
        double r;
        if (i < N / 2) r = (1.0 + CFL) * fl[q] - CFL * fl[q + n3];
        else r = (1.0 - CFL) * fl[q] + CFL * fl[q - n3];
        if (ic == 5) {  // Poiseuille forcing, Ma = 1 (transportroutines.c:218-225)
            const double c = 1.0 * dt / (2 * dx[l]);
            if (j == 0) r = r - c * fl[q + N];
            else if (j == N - 1) r = r - c * fl[q - N];
            else r = r - c * (fl[q + N] - fl[q - N]);
        }
        fc[(long long)l * n3 + q] = r;
    }
}

__device__ __forceinline__ double slope_at(const double *f, const double *x, int l,
                                           long long q, long long n3)
{
    // minmod slope of cell l (transportroutines.c:388-390)
    const double fm = f[(long long)(l - 1) * n3 + q], f0 = f[(long long)l * n3 + q],
                 fp = f[(long long)(l + 1) * n3 + q];
    return minmod3((f0 - fm) / (x[l] - x[l - 1]), (fp - f0) / (x[l + 1] - x[l]),
                   (fp - fm) / (x[l + 1] - x[l - 1]));
}

// Wall values of upwindTwo (transportroutines.c:366-431): f_l from cell 2,
// f_r from cell nX+1.  For diffuse or heated walls only the outgoing half
// is set here; the wall kernel then fills the incoming half.
__global__ void wall_values_kernel(const double *__restrict__ f, double *__restrict__ f_l,
                                   double *__restrict__ f_r, const double *__restrict__ x,
                                   const double *__restrict__ dx, int N, int nX, int ic)
{
    const long long n3 = (long long)N * N * N;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < 2 * n3;
         t += (long long)gridDim.x * blockDim.x) {
        const bool right = t >= n3;
        const long long q = right ? t - n3 : t;
        const int i = (int)q / (N * N);
        const bool upper = i >= N / 2;
        if (!right) {
            const double s1 = slope_at(f, x, 2, q, n3);
            const double f2 = f[2 * n3 + q];
            if (!upper) f_l[q] = f2 - 0.5 * dx[2] * s1;
            else if (!(ic == 3 || ic == 5 || ic == 1)) f_l[q] = f2 + 0.5 * dx[2] * s1;
        } else {
            const double s1 = slope_at(f, x, nX + 1, q, n3);
            const double fn = f[(long long)(nX + 1) * n3 + q];
            if (upper) f_r[q] = fn + 0.5 * dx[nX + 1] * s1;
            else if (!(ic == 3 || ic == 5)) f_r[q] = fn - 0.5 * dx[nX + 1] * s1;
        }
    }
}

// Second-order minmod upwind for cells 2..nX+1 (transportroutines.c:433-469).
__global__ void upwind2_kernel(const double *__restrict__ f, double *__restrict__ fc,
                               const double *__restrict__ f_l, const double *__restrict__ f_r,
                               const double *__restrict__ v, const double *__restrict__ x,
                               const double *__restrict__ dx, int N, int nX, double dt, int ic)
{
    const long long n3 = (long long)N * N * N;
    const long long total = (long long)nX * n3;
    const double h_v = v[1] - v[0];
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const unsigned tc = (unsigned)t / (unsigned)n3;  // 32-bit: nX N^3 < 2^31
        const int l = 2 + (int)tc;
        const long long q = (long long)((unsigned)t - tc * (unsigned)n3);
        const int i = (int)q / (N * N), j = ((int)q / N) % N;
        const double *fl = f + (long long)l * n3;
        const double CFL = 0.5 * dt * v[i] / dx[l];
        double r;
        if (i >= N / 2) {
            const double s1 = slope_at(f, x, l, q, n3);
            if (l == 2) {
                r = fl[q] - CFL * (fl[q] + 0.5 * dx[l] * s1 - f_l[q]);
            } else {
                const double s0 = slope_at(f, x, l - 1, q, n3);
                r = fl[q] - CFL * (fl[q] + 0.5 * dx[l] * s1 - (fl[q - n3] + 0.5 * dx[l - 1] * s0));
            }
        } else {
            const double s1 = slope_at(f, x, l, q, n3);
            if (l == nX + 1) {
                r = fl[q] - CFL * (f_r[q] - (fl[q] - 0.5 * dx[l] * s1));
            } else {
                const double s2 = slope_at(f, x, l + 1, q, n3);
                r = fl[q] - CFL * (fl[q + n3] - 0.5 * dx[l + 1] * s2 - (fl[q] - 0.5 * dx[l] * s1));
            }
        }
        if (ic == 5) {  // Poiseuille forcing, Ma = 1 (transportroutines.c:407-414)
            const double c = 1.0 * 0.5 * dt / (2 * h_v);
            if (j == 0) r = r - c * fl[q + N];
            else if (j == N - 1) r = r - c * fl[q - N];
            else r = r - c * (fl[q + N] - fl[q - N]);
        }
        fc[(long long)l * n3 + q] = r;
    }
}

// Ghost cells of upwindTwo on one rank (transportroutines.c:273-300):
// f[1] = 2 f[2] - f[3], f[nX+2] = 2 f[nX+1] - f[nX].  The outer ghosts
// f[0], f[nX+3] are not filled by the reference and only reach slopes that
// are never used; they are set to the inner ghosts so every value is finite.
__global__ void ghosts2_kernel(double *__restrict__ f, int N, int nX)
{
    const long long n3 = (long long)N * N * N;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n3;
         q += (long long)gridDim.x * blockDim.x) {
        const double g1 = 2 * f[2 * n3 + q] - f[3 * n3 + q];
        const double g2 = 2 * f[(long long)(nX + 1) * n3 + q] - f[(long long)nX * n3 + q];
        f[n3 + q] = g1;
        f[q] = g1;
        f[(long long)(nX + 2) * n3 + q] = g2;
        f[(long long)(nX + 3) * n3 + q] = g2;
    }
}

int grid_for(long long n)
{
    long long b = (n + 255) / 256;
    if (b > 152 * 16) b = 152 * 16;
    return (int)(b < 1 ? 1 : b);
}

}  // namespace

cudaError_t transport_ghosts1(double *f, const double *v, const TransportParams &tp,
                              cudaStream_t st)
{
    // ghost cells of upwindOne on one rank (transportroutines.c:116-172)
    const int N = tp.N, nX = tp.nX, ic = tp.ic;
    const long long n3 = (long long)N * N * N;
    double *F0 = f, *F1 = f + n3, *Fn = f + (long long)nX * n3, *Fn1 = f + (long long)(nX + 1) * n3;
    BcJob jobs[2];
    int nj = 0;
    cudaError_t e = cudaSuccess;
    if (ic == 3 || ic == 5) jobs[nj++] = BcJob{F1, F0, tp.T0, 0};
    else if (ic == 1) jobs[nj++] = BcJob{F1, F0, 2.0 * tp.TWall, 0};
    else if (ic != 6) e = cudaMemcpyAsync(F0, F1, sizeof(double) * n3, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    if (ic == 3 || ic == 5) jobs[nj++] = BcJob{Fn, Fn1, tp.T1, 1};
    else if (ic != 6) e = cudaMemcpyAsync(Fn1, Fn, sizeof(double) * n3, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return e;
    if (ic == 6) {  // periodic on one rank
        e = cudaMemcpyAsync(F0, Fn, sizeof(double) * n3, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(Fn1, F1, sizeof(double) * n3, cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return e;
    }
    if (nj) {
        diffuse_bc_kernel<<<nj, 256, 0, st>>>(jobs[0], nj > 1 ? jobs[1] : jobs[0], nj, v, N,
                                              tp.mass, tp.KB);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t transport_upwind1(const double *f, double *fc, const double *v, const double *dx,
                              const TransportParams &tp, cudaStream_t st)
{
    const long long n = (long long)tp.nX * tp.N * tp.N * tp.N;
    upwind1_kernel<<<grid_for(n), 256, 0, st>>>(f, fc, v, dx, tp.N, tp.nX, tp.dt, tp.ic);
    return cudaGetLastError();
}

cudaError_t transport_upwind2(double *f, double *fc, double *f_l, double *f_r, const double *v,
                              const double *x, const double *dx, const TransportParams &tp,
                              cudaStream_t st)
{
    const int N = tp.N, nX = tp.nX, ic = tp.ic;
    const long long n3 = (long long)N * N * N;
    ghosts2_kernel<<<grid_for(n3), 256, 0, st>>>(f, N, nX);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    wall_values_kernel<<<grid_for(2 * n3), 256, 0, st>>>(f, f_l, f_r, x, dx, N, nX, ic);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    BcJob jobs[2];
    int nj = 0;
    if (ic == 3 || ic == 5) jobs[nj++] = BcJob{f_l, f_l, tp.T0, 0};
    else if (ic == 1) jobs[nj++] = BcJob{f_l, f_l, 2.0 * tp.TWall, 0};
    if (ic == 3 || ic == 5) jobs[nj++] = BcJob{f_r, f_r, tp.T1, 1};
    if (nj) {
        diffuse_bc_kernel<<<nj, 256, 0, st>>>(jobs[0], nj > 1 ? jobs[1] : jobs[0], nj, v, N,
                                              tp.mass, tp.KB);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    upwind2_kernel<<<grid_for((long long)nX * n3), 256, 0, st>>>(f, fc, f_l, f_r, v, x, dx, N,
                                                                 nX, tp.dt, ic);
    return cudaGetLastError();
}

}  // namespace sbte
