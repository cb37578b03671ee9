/*
 * spectral_oracle.c -- CPU restatement of the SpectralBTE collision path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT.  It checks and times the GPU library and
 * never runs inside it.  See spectral_oracle.h for the conventions.
 *
 * Build with -ffp-contract=off so that x86 and aarch64 round the same way.
 * Expressions keep the reference's operand order.
 */
#include "spectral_oracle.h"
#include "dft3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static void trap_weights(int N, double *wt)
{
    /* collisions.c:48-54, conserve.c:35-39, momentRoutines.c:14-18 */
    wt[0] = 0.5;
    for (int i = 1; i < N - 1; i++) wt[i] = 1.0;
    wt[N - 1] = 0.5;
}

/* ------------------------------------------------------------------ grids */
void oracle_grid_0d(int N, double L_v, double *v, double *zeta)
{
    /* initializer.c:66-82 */
    double dv = 2 * L_v / (N - 1);
    for (int i = 0; i < N; i++) v[i] = -L_v + i * dv;
    double deta = (2 * M_PI / N) / dv;
    double L_eta = ((N % 2) == 0) ? 0.5 * N * deta : 0.5 * (N - 1) * deta;
    for (int i = 0; i < N; i++) zeta[i] = -L_eta + i * deta;
}

void oracle_grid_1d(int N, double L_v, double *v, double *zeta)
{
    /* initializer.c:256-266 */
    double dv = 2 * L_v / (N - 1);
    for (int i = 0; i < N; i++) v[i] = -L_v + i * dv;
    double L_eta = 0.5 * (N - 1) * M_PI / L_v;
    double deta = M_PI * (N - 1) / (N * L_v);
    for (int i = 0; i < N; i++) zeta[i] = -L_eta + i * deta;
}

/* -------------------------------------------------------------------- FFT */
void oracle_fft3d(int N, double L_v, const double *v, const double *eta,
                  const double *in, double *out, int invert)
{
    /* Module state of initialize_coll, collisions.c:36-46. */
    double dv = v[1] - v[0];
    double deta = eta[1] - eta[0];
    double L_eta = -eta[0];
    double scale3 = pow(1.0 / sqrt(2.0 * M_PI), 3.0);
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);

    double delta, L_start, L_end, sign;
    const double *varr;
    int dir;
    if (!invert) { /* collisions.c:238-245 */
        delta = dv; L_start = L_eta; L_end = L_v; varr = eta; sign = 1.0;
        dir = -1; /* FFTW_FORWARD */
    } else {       /* collisions.c:246-253 */
        delta = deta; L_start = L_v; L_end = L_eta; varr = v; sign = -1.0;
        dir = +1; /* FFTW_BACKWARD */
    }
    double prefactor = scale3 * delta * delta * delta;
    long n3 = (long)N * N * N;
    double *temp = (double *)malloc(sizeof(double) * 2 * n3);

    /* pre-shift, collisions.c:257-268 */
    for (long index = 0; index < n3; index++) {
        int i = (int)(index / ((long)N * N));
        int j = (int)((index - (long)i * N * N) / N);
        int k = (int)(index - (long)N * (j + (long)i * N));
        double sum = sign * (double)(i + j + k) * L_start * delta;
        double factor = prefactor * wtN[i] * wtN[j] * wtN[k];
        double c = cos(sum), s = sin(sum);
        temp[2 * index] = factor * (c * in[2 * index] - s * in[2 * index + 1]);
        temp[2 * index + 1] =
            factor * (c * in[2 * index + 1] + s * in[2 * index]);
    }
    /* fftw_execute, collisions.c:270 */
    oracle_dft3(N, N, N, temp, dir);
    /* post-shift, collisions.c:273-281 */
    for (long index = 0; index < n3; index++) {
        int i = (int)(index / ((long)N * N));
        int j = (int)((index - (long)i * N * N) / N);
        int k = (int)(index - (long)N * (j + (long)i * N));
        double sum = sign * L_end * (varr[i] + varr[j] + varr[k]);
        double c = cos(sum), s = sin(sum);
        double tr = temp[2 * index], ti = temp[2 * index + 1];
        out[2 * index] = c * tr - s * ti;
        out[2 * index + 1] = c * ti + s * tr;
    }
    free(temp);
    free(wtN);
}

/* ------------------------------------------------------------ convolution */
void oracle_compute_qhat(int N, double L_v, const double *v,
                         const double *zeta, const double *W,
                         const double *f, const double *g, double *q,
                         double *fhat_out, double *ghat_out,
                         double *qhat_out, int nthreads)
{
    long n3 = (long)N * N * N;
    double *fin = (double *)malloc(sizeof(double) * 2 * n3);
    double *gin = (double *)malloc(sizeof(double) * 2 * n3);
    double *fo = (double *)malloc(sizeof(double) * 2 * n3);
    double *go = (double *)malloc(sizeof(double) * 2 * n3);
    double *qh = (double *)malloc(sizeof(double) * 2 * n3);
    /* collisions.c:112-119 */
    for (long index = 0; index < n3; index++) {
        qh[2 * index] = 0.0; qh[2 * index + 1] = 0.0;
        fin[2 * index] = f[index]; fin[2 * index + 1] = 0.0;
        gin[2 * index] = g[index]; gin[2 * index + 1] = 0.0;
    }
    /* collisions.c:122-123 */
    oracle_fft3d(N, L_v, v, zeta, fin, fo, 0);
    oracle_fft3d(N, L_v, v, zeta, gin, go, 0);

    /* collisions.c:127-165: rows of zeta in parallel, xi sequential */
    int n2 = N / 2;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(static)
#else
    (void)nthreads;
#endif
    for (long zeta_i = 0; zeta_i < n3; zeta_i++) {
        int zx = (int)(zeta_i / ((long)N * N));
        int zy = (int)((zeta_i - (long)zx * N * N) / N);
        int zz = (int)(zeta_i - (long)N * (zy + (long)zx * N));
        const double *row = W + zeta_i * n3;
        double acc_re = 0.0, acc_im = 0.0;
        for (long xi = 0; xi < n3; xi++) {
            int xx = (int)(xi / ((long)N * N));
            int xy = (int)((xi - (long)xx * N * N) / N);
            int xz = (int)(xi - (long)N * (xy + (long)xx * N));
            int x = zx + n2 - xx, y = zy + n2 - xy, z = zz + n2 - xz;
            if (x < 0) x = N + x; else if (x > N - 1) x = x - N;
            if (y < 0) y = N + y; else if (y > N - 1) y = y - N;
            if (z < 0) z = N + z; else if (z > N - 1) z = z - N;
            long index = z + (long)N * (y + (long)N * x);
            acc_re += row[xi] * (go[2 * xi] * fo[2 * index] -
                                 go[2 * xi + 1] * fo[2 * index + 1]);
            acc_im += row[xi] * (go[2 * xi] * fo[2 * index + 1] +
                                 go[2 * xi + 1] * fo[2 * index]);
        }
        qh[2 * zeta_i] = acc_re;
        qh[2 * zeta_i + 1] = acc_im;
    }
    if (fhat_out) memcpy(fhat_out, fo, sizeof(double) * 2 * n3);
    if (ghat_out) memcpy(ghat_out, go, sizeof(double) * 2 * n3);
    if (qhat_out) memcpy(qhat_out, qh, sizeof(double) * 2 * n3);
    if (q) {
        /* collisions.c:168 then :218-220 */
        oracle_fft3d(N, L_v, v, zeta, qh, fo, 1);
        for (long index = 0; index < n3; index++) q[index] = fo[2 * index];
    }
    free(fin); free(gin); free(fo); free(go); free(qh);
}

void oracle_qhat_rows(int N, const double *W_rows, int row0, int nrows,
                      const double *fo, const double *go, double *qh,
                      int nthreads)
{
    /* collisions.c:127-165 restricted to zeta in [row0, row0+nrows) */
    long n3 = (long)N * N * N;
    int n2 = N / 2;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(static)
#else
    (void)nthreads;
#endif
    for (long r = 0; r < nrows; r++) {
        long zeta_i = row0 + r;
        int zx = (int)(zeta_i / ((long)N * N));
        int zy = (int)((zeta_i - (long)zx * N * N) / N);
        int zz = (int)(zeta_i - (long)N * (zy + (long)zx * N));
        const double *row = W_rows + r * n3;
        double acc_re = 0.0, acc_im = 0.0;
        for (long xi = 0; xi < n3; xi++) {
            int xx = (int)(xi / ((long)N * N));
            int xy = (int)((xi - (long)xx * N * N) / N);
            int xz = (int)(xi - (long)N * (xy + (long)xx * N));
            int x = zx + n2 - xx, y = zy + n2 - xy, z = zz + n2 - xz;
            if (x < 0) x = N + x; else if (x > N - 1) x = x - N;
            if (y < 0) y = N + y; else if (y > N - 1) y = y - N;
            if (z < 0) z = N + z; else if (z > N - 1) z = z - N;
            long index = z + (long)N * (y + (long)N * x);
            acc_re += row[xi] * (go[2 * xi] * fo[2 * index] - go[2 * xi + 1] * fo[2 * index + 1]);
            acc_im += row[xi] * (go[2 * xi] * fo[2 * index + 1] + go[2 * xi + 1] * fo[2 * index]);
        }
        qh[2 * r] = acc_re;
        qh[2 * r + 1] = acc_im;
    }
}

void oracle_computeQ(int N, double L_v, const double *v, const double *zeta,
                     const double *W, const double *f, const double *g,
                     double *Q, int nthreads)
{
    oracle_compute_qhat(N, L_v, v, zeta, W, f, g, Q, NULL, NULL, NULL,
                        nthreads);
}

/* ---------------------------------------------------------------- moments */
double oracle_density(int N, const double *v, const double *in, double mass)
{
    /* momentRoutines.c:58-69 */
    double dv = v[1] - v[0], dv3 = dv * dv * dv, result = 0.0;
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++)
                result += dv3 * wtN[i] * wtN[j] * wtN[k] * in[k + N * (j + N * i)];
    free(wtN);
    return mass * result;
}

void oracle_bulk_velocity(int N, const double *v, const double *in,
                          double rho, double mass, double *out)
{
    /* momentRoutines.c:116-141 */
    double dv = v[1] - v[0], dv3 = dv * dv * dv;
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);
    out[0] = out[1] = out[2] = 0.0;
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                double t1 = v[i] * dv3 * wtN[i] * wtN[j] * wtN[k] / rho;
                double t2 = v[j] * dv3 * wtN[i] * wtN[j] * wtN[k] / rho;
                double t3 = v[k] * dv3 * wtN[i] * wtN[j] * wtN[k] / rho;
                double x = in[k + N * (j + N * i)];
                out[0] += t1 * x; out[1] += t2 * x; out[2] += t3 * x;
            }
    out[0] = mass * out[0]; out[1] = mass * out[1]; out[2] = mass * out[2];
    free(wtN);
}

double oracle_temperature(int N, const double *v, const double *in,
                          const double *bulkV, double rho, double mass,
                          double KB)
{
    /* momentRoutines.c:168-183 */
    double dv = v[1] - v[0], dv3 = dv * dv * dv, result = 0.0;
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                double temp = (v[i] - bulkV[0]) * (v[i] - bulkV[0]) +
                              (v[j] - bulkV[1]) * (v[j] - bulkV[1]) +
                              (v[k] - bulkV[2]) * (v[k] - bulkV[2]);
                result += temp * dv3 * wtN[i] * wtN[j] * wtN[k] *
                          in[k + N * (j + N * i)] / (3.0 * rho);
            }
    free(wtN);
    return (mass * mass / KB) * result;
}

void oracle_energy(int N, const double *v, const double *in, double *out)
{
    /* momentRoutines.c:146-165 */
    double dv = v[1] - v[0], dv3 = dv * dv * dv, pos = 0.0, neg = 0.0;
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                double e = dv3 * wtN[i] * wtN[j] * wtN[k] * in[k + N * (j + N * i)] *
                           (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
                if (e > 0) pos += e; else neg -= e;
            }
    out[0] = pos; out[1] = neg;
    free(wtN);
}

/* --------------------------------------------------------- maxPreserve */
static void find_maxwellian(int N, const double *v, const double *mat,
                            double mass, double KB, double *M)
{
    /* collisions.c:95-103 (the g part is formed by the caller) */
    double vel[3];
    double rho = oracle_density(N, v, mat, mass);
    oracle_bulk_velocity(N, v, mat, rho, mass, vel);
    double T = oracle_temperature(N, v, mat, vel, rho, mass, KB);
    double prefactor = rho * pow(0.5 / (M_PI * T), 1.5);
    for (long index = 0; index < (long)N * N * N; index++) {
        int i = (int)(index / (N * N));
        int j = (int)((index - (long)i * N * N) / N);
        int k = (int)(index - (long)N * (j + (long)N * i));
        M[index] = prefactor * exp(-(0.5 / T) * ((v[i] - vel[0]) * (v[i] - vel[0]) +
                                                 (v[j] - vel[1]) * (v[j] - vel[1]) +
                                                 (v[k] - vel[2]) * (v[k] - vel[2])));
    }
}

void oracle_computeQ_maxPreserve(int N, double L_v, const double *v,
                                 const double *zeta, const double *W,
                                 const double *f, const double *g, double *Q,
                                 double mass, double KB, int nthreads)
{
    long n3 = (long)N * N * N;
    double *Mi = (double *)malloc(sizeof(double) * n3);
    double *Mj = (double *)malloc(sizeof(double) * n3);
    double *gi = (double *)malloc(sizeof(double) * n3);
    double *gj = (double *)malloc(sizeof(double) * n3);
    double *t = (double *)malloc(sizeof(double) * n3);
    /* collisions.c:181-182; both g's subtract M_i (collisions.c:104) */
    find_maxwellian(N, v, f, mass, KB, Mi);
    for (long x = 0; x < n3; x++) gi[x] = f[x] - Mi[x];
    find_maxwellian(N, v, g, mass, KB, Mj);
    for (long x = 0; x < n3; x++) gj[x] = g[x] - Mi[x];
    /* collisions.c:184-200 */
    oracle_compute_qhat(N, L_v, v, zeta, W, Mi, gj, t, 0, 0, 0, nthreads);
    for (long x = 0; x < n3; x++) Q[x] = t[x];
    oracle_compute_qhat(N, L_v, v, zeta, W, gi, Mj, t, 0, 0, 0, nthreads);
    for (long x = 0; x < n3; x++) Q[x] += t[x];
    oracle_compute_qhat(N, L_v, v, zeta, W, gi, gj, t, 0, 0, 0, nthreads);
    for (long x = 0; x < n3; x++) Q[x] += t[x];
    free(Mi); free(Mj); free(gi); free(gj); free(t);
}

/* ----------------------------------------------------------- conservation */
static int factor_lu(oracle_cons *c, int nElem)
{
    /* factorMatrixIntoLU, conserve.c:89-168 (scaled pivoting after
       Atkinson; the pivot row is the first row whose scaled entry beats the
       running best, and only columns >= k are exchanged). */
    double s[ORACLE_MAX_NS + 4], cc[ORACLE_MAX_NS + 4], m[ORACLE_MAX_NS + 4];
    for (int i = 0; i < nElem; i++) {
        s[i] = fabs(c->CCt[i][0]);
        for (int j = 0; j < nElem; j++)
            if (s[i] < fabs(c->CCt[i][j])) s[i] = fabs(c->CCt[i][j]);
    }
    for (int k = 0; k < nElem - 1; k++) {
        cc[k] = fabs(c->CCt[k][k] / s[k]);
        int ctr = 0, i0 = k;
        for (int i = k; i < nElem; i++) {
            if (cc[k] < fabs(c->CCt[i][k] / s[i])) {
                cc[k] = fabs(c->CCt[i][k] / s[i]);
                if (ctr != 1) { i0 = i; ctr = 1; }
            }
        }
        c->pivot[k] = i0;
        if (cc[k] == 0.0) return -1;
        if (i0 != k) {
            for (int j = k; j < nElem; j++) {
                double t = c->CCt[k][j];
                c->CCt[k][j] = c->CCt[i0][j];
                c->CCt[i0][j] = t;
            }
            double t = s[k]; s[k] = s[i0]; s[i0] = t;
        }
        for (int i = k + 1; i < nElem; i++) {
            m[i] = c->CCt[i][k] / c->CCt[k][k];
            c->CCt[i][k] = m[i];
            for (int j = k + 1; j < nElem; j++) c->CCt[i][j] -= m[i] * c->CCt[k][j];
        }
    }
    return 0;
}

int oracle_conservation_init(oracle_cons *c, int N, double dv,
                             const double *v, const double *mass, int Ns)
{
    /* initialize_conservation + createCCtAndPivot, conserve.c:17-43, 268-317 */
    memset(c, 0, sizeof(*c));
    c->N = N; c->Ns = Ns; c->dv = dv; c->v = v;
    for (int m = 0; m < Ns; m++) c->mass[m] = mass[m];
    int ne = Ns + 4;
    long n3 = (long)N * N * N;
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);
    /* C[m][row][x] */
    double *C = (double *)calloc((size_t)Ns * ne * n3, sizeof(double));
    for (int m = 0; m < Ns; m++)
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++)
                for (int k = 0; k < N; k++) {
                    long x = k + N * (j + (long)N * i);
                    double prefactor = wtN[i] * wtN[j] * wtN[k] * dv * dv * dv * mass[m];
                    double *Cm = C + (long)m * ne * n3;
                    for (int n = 0; n < Ns; n++) Cm[n * n3 + x] = 0;
                    Cm[m * n3 + x] = prefactor;
                    Cm[(Ns) * n3 + x] = prefactor * v[i];
                    Cm[(Ns + 1) * n3 + x] = prefactor * v[j];
                    Cm[(Ns + 2) * n3 + x] = prefactor * v[k];
                    Cm[(Ns + 3) * n3 + x] =
                        prefactor * 0.5 * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
                }
    for (int i = 0; i < ne; i++)
        for (int j = 0; j < ne; j++) {
            double acc = 0.0;
            for (int m = 0; m < Ns; m++) {
                const double *Cm = C + (long)m * ne * n3;
                for (long k = 0; k < n3; k++) acc += Cm[i * n3 + k] * Cm[j * n3 + k];
            }
            c->CCt[i][j] = acc;
        }
    free(C);
    free(wtN);
    return factor_lu(c, ne);
}

void oracle_solve_cct(const oracle_cons *c, double *b)
{
    /* solveWithCCt, conserve.c:173-202 */
    int nElem = c->Ns + 4;
    for (int k = 0; k < nElem - 1; k++) {
        int i = c->pivot[k];
        if (c->pivot[k] != k) { double t = b[i]; b[i] = b[k]; b[k] = t; }
        for (i = k + 1; i < nElem; i++) b[i] -= c->CCt[i][k] * b[k];
    }
    b[nElem - 1] = b[nElem - 1] / c->CCt[nElem - 1][nElem - 1];
    for (int i = nElem - 2; i >= 0; i--) {
        double sum = 0.0;
        for (int j = i + 1; j < nElem; j++) sum += c->CCt[i][j] * b[j];
        b[i] = 1.0 / c->CCt[i][i] * (b[i] - sum);
    }
}

void oracle_conserve(const oracle_cons *c, double **Q)
{
    /* conserveAllMoments, conserve.c:207-264 */
    int N = c->N, Ns = c->Ns;
    double dv = c->dv;
    const double *v = c->v;
    double masterQ[ORACLE_MAX_NS + 4], tc[ORACLE_MAX_NS + 4];
    double wtN[4096];
    trap_weights(N, wtN);
    for (int l = 0; l < Ns + 4; l++) masterQ[l] = 0.0;
    memset(tc, 0, sizeof(tc));
    for (int m = 0; m < Ns; m++)
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++)
                for (int k = 0; k < N; k++) {
                    double prefact = wtN[i] * wtN[j] * wtN[k] * dv * dv * dv * c->mass[m];
                    tc[m] = prefact;
                    tc[Ns] = prefact * v[i];
                    tc[Ns + 1] = prefact * v[j];
                    tc[Ns + 2] = prefact * v[k];
                    tc[Ns + 3] = prefact * 0.5 * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
                    long x = k + N * (j + (long)N * i);
                    for (int n = 0; n < Ns; n++) {
                        double q = Q[n * Ns + m][x];
                        masterQ[m] += q * tc[m];
                        masterQ[Ns] += q * tc[Ns];
                        masterQ[Ns + 1] += q * tc[Ns + 1];
                        masterQ[Ns + 2] += q * tc[Ns + 2];
                        masterQ[Ns + 3] += q * tc[Ns + 3];
                    }
                }
    oracle_solve_cct(c, masterQ);
    for (int m = 0; m < Ns; m++)
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++)
                for (int k = 0; k < N; k++) {
                    double prefact = wtN[i] * wtN[j] * wtN[k] * dv * dv * dv * c->mass[m] / Ns;
                    tc[m] = prefact;
                    tc[Ns] = prefact * v[i];
                    tc[Ns + 1] = prefact * v[j];
                    tc[Ns + 2] = prefact * v[k];
                    tc[Ns + 3] = prefact * 0.5 * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]);
                    long x = k + N * (j + (long)N * i);
                    for (int n = 0; n < Ns; n++)
                        Q[n * Ns + m][x] -= (tc[m] * masterQ[m] + tc[Ns] * masterQ[Ns] +
                                             tc[Ns + 1] * masterQ[Ns + 1] +
                                             tc[Ns + 2] * masterQ[Ns + 2] +
                                             tc[Ns + 3] * masterQ[Ns + 3]);
                }
}

void oracle_conserve_batch1(const oracle_cons *c, double *Q, int B)
{
    long n3 = (long)c->N * c->N * c->N;
    for (int b = 0; b < B; b++) {
        double *p = Q + (long)b * n3;
        oracle_conserve(c, &p);
    }
}

/* ------------------------------------------------------------- quadrature */
void oracle_gauss_legendre(int n, double *x, double *w)
{
    /* Newton iteration on the three-term Legendre recurrence
       (k+1) P_{k+1} = (2k+1) x P_k - k P_{k-1}, started from
       cos(pi (i - 1/4) / (n + 1/2)); w = 2 / ((1 - x^2) P_n'(x)^2).
       Nodes come out in decreasing order and are stored ascending. */
    for (int i = 1; i <= (n + 1) / 2; i++) {
        double z = cos(M_PI * (i - 0.25) / (n + 0.5)), pp = 0.0;
        for (int it = 0; it < 100; it++) {
            double p1 = 1.0, p2 = 0.0;
            for (int k = 1; k <= n; k++) {
                double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * k - 1.0) * z * p2 - (k - 1.0) * p3) / k;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.0);
            double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) <= 1e-16) {
                /* one more evaluation at the converged node */
                p1 = 1.0; p2 = 0.0;
                for (int k = 1; k <= n; k++) {
                    double p3 = p2;
                    p2 = p1;
                    p1 = ((2.0 * k - 1.0) * z * p2 - (k - 1.0) * p3) / k;
                }
                pp = n * (z * p1 - p2) / (z * z - 1.0);
                break;
            }
        }
        x[n - i] = z;
        x[i - 1] = -z;
        w[i - 1] = w[n - i] = 2.0 / ((1.0 - z * z) * pp * pp);
    }
}

#define ORACLE_GL_POINTS 16
int oracle_quad_panels(double L_v, double omega)
{
    /* With 16 nodes per panel and omega*h <= 6 rad, the truncation error of
       a panel is below (3)^32/32! ~ 1e-20 of the integrand scale. */
    int K = (int)ceil(omega * L_v / 6.0);
    if (K < 4) K = 4;
    return K;
}

static double sinc_ref(double x)
{
    /* weights.c:136-143 */
    return (x != 0.0) ? sin(x) / x : 1.0;
}

double oracle_ghat_integral(double a0, double a1, double a2, double lambda,
                            double L_v)
{
    /* Integral of ghat (weights.c:156-160) over [0, L_v]; the reference uses
       gsl_integration_qag with the 21-point rule to 1e-8 (weights.c:203).
       This uses composite 16-point Gauss-Legendre, converged to round-off. */
    static double gx[ORACLE_GL_POINTS], gw[ORACLE_GL_POINTS];
    static int init = 0;
    if (!init) {
#ifdef _OPENMP
#pragma omp critical(oracle_gl_init)
#endif
        {
            if (!init) { oracle_gauss_legendre(ORACLE_GL_POINTS, gx, gw); init = 1; }
        }
    }
    double omega = a0 + a2 > a1 ? a0 + a2 : a1;
    int K = oracle_quad_panels(L_v, omega);
    double h = L_v / K, result = 0.0;
    for (int p = 0; p < K; p++) {
        double mid = (p + 0.5) * h, part = 0.0;
        for (int q = 0; q < ORACLE_GL_POINTS; q++) {
            double r = mid + 0.5 * h * gx[q];
            double val = pow(r, lambda + 2) *
                         (sinc_ref(r * a0) * sinc_ref(r * a2) - sinc_ref(r * a1));
            part += gw[q] * val;
        }
        result += 0.5 * h * part;
    }
    return result;
}

/* Closed forms of the radial integral of ghat (weights.c:156-160) for
   lambda = 0 and 1, derived here from the integrand (the reference
   integrates it numerically, weights.c:203).  With s(x) = sin x / x and
   q(x) = (1 - cos x) / x^2 = s(x/2)^2 / 2 (no cancellation at small x):
     gain, lambda = 0:  int_0^L r^2 s(ra) s(rb) dr = L / (2ab) [s(Ld) - s(Le)]
     gain, lambda = 1:  int_0^L r^3 s(ra) s(rb) dr
                          = L^2 / (2ab) [s(Ld) - q(Ld) - s(Le) + q(Le)]
       with d = a - b, e = a + b (from 2 sin A sin B = cos(A-B) - cos(A+B)
       and int_0^L r cos(rk) dr = L^2 [s(Lk) - q(Lk)]);
     loss, lambda = 0:  int_0^L r^2 s(rc) dr = (sin x - x cos x) / c^3
     loss, lambda = 1:  int_0^L r^3 s(rc) dr = ((2 - x^2) cos x + 2x sin x - 2) / c^4
       with x = Lc; below x = 1/2 the loss uses its series
       L^(lambda+3) sum_k (-1)^k x^(2k) / ((2k+1)! (2k+lambda+3)).
   A gain argument of exactly 0 turns the gain into the loss form of the
   other argument (s = 1).  A gain argument that is nonzero but below 1/2 / L
   would lose digits in 1/(ab): such entries (none on the grids of this
   project) and every other lambda use the quadrature. */
static double loss_closed(double c, int lam, double L)
{
    const double x = L * c;
    const double Lp = lam == 0 ? L * L * L : L * L * L * L;
    if (x < 0.5) {
        double term = 1.0, sum = 0.0;  /* term = (-1)^k x^(2k) / (2k+1)! */
        for (int k = 0; k < 12; k++) {
            sum += term / (2.0 * k + lam + 3.0);
            term *= -x * x / ((2.0 * k + 2.0) * (2.0 * k + 3.0));
        }
        return Lp * sum;
    }
    const double sx = sin(x), cx = cos(x);
    if (lam == 0) return (sx - x * cx) / (c * c * c);
    return ((2.0 - x * x) * cx + 2.0 * x * sx - 2.0) / (c * c * c * c);
}

static double q_stable(double x)
{
    const double h = sinc_ref(0.5 * x);
    return 0.5 * h * h;
}

double oracle_ghat_closed(double a0, double a1, double a2, double lambda, double L_v)
{
    const int lam = (lambda == 0.0) ? 0 : (lambda == 1.0 ? 1 : -1);
    const double small = 0.5 / L_v;
    if (lam < 0 || (a0 != 0.0 && a0 < small) || (a2 != 0.0 && a2 < small))
        return oracle_ghat_integral(a0, a1, a2, lambda, L_v);
    double gain;
    if (a0 == 0.0 && a2 == 0.0)
        gain = (lam == 0 ? L_v * L_v * L_v / 3.0 : L_v * L_v * L_v * L_v / 4.0);
    else if (a0 == 0.0)
        gain = loss_closed(a2, lam, L_v);
    else if (a2 == 0.0)
        gain = loss_closed(a0, lam, L_v);
    else {
        const double d = L_v * (a0 - a2), e = L_v * (a0 + a2);
        if (lam == 0)
            gain = L_v / (2.0 * a0 * a2) * (sinc_ref(d) - sinc_ref(e));
        else
            gain = L_v * L_v / (2.0 * a0 * a2) *
                   (sinc_ref(d) - q_stable(d) - sinc_ref(e) + q_stable(e));
    }
    return gain - loss_closed(a1, lam, L_v);
}

static void weights_iso_rows(int N, const double *zeta, double L_v, double lambda,
                             double d_i, double d_j, double m_i, double m_j,
                             int row_begin, int row_end, double *W, int nthreads, int closed)
{
    /* initialize_weights (weights.c:41-49) and generate_conv_weights_iso
       (weights.c:265-281) with gHat3 (weights.c:181-262) */
    double deta = zeta[1] - zeta[0];
    double prefactor = 16.0 * M_PI * M_PI * deta * deta * deta / pow(2.0 * M_PI, 1.5) / (4.0 * M_PI);
    double mu = m_j / (m_i + m_j);
    double *wtN = (double *)malloc(sizeof(double) * N);
    trap_weights(N, wtN);
    long n3 = (long)N * N * N;
    double dfac = 0.25 * pow(0.5 * (d_i + d_j), 2);
    (void)dfac;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for num_threads(nt) schedule(dynamic)
#else
    (void)nthreads;
#endif
    for (long row = row_begin; row < row_end; row++) {
        int i = (int)(row / ((long)N * N));
        int j = (int)((row / N) % N);
        int k = (int)(row % N);
        double z1 = zeta[i], z2 = zeta[j], z3 = zeta[k];
        for (long col = 0; col < n3; col++) {
            int l = (int)(col / ((long)N * N));
            int m = (int)((col / N) % N);
            int n = (int)(col % N);
            double k1 = zeta[l], k2 = zeta[m], k3 = zeta[n];
            double a0 = mu * sqrt(z1 * z1 + z2 * z2 + z3 * z3);
            double a1 = sqrt(k1 * k1 + k2 * k2 + k3 * k3);
            double a2 = sqrt((k1 - mu * z1) * (k1 - mu * z1) + (k2 - mu * z2) * (k2 - mu * z2) +
                             (k3 - mu * z3) * (k3 - mu * z3));
            double g = prefactor * (closed ? oracle_ghat_closed(a0, a1, a2, lambda, L_v)
                                           : oracle_ghat_integral(a0, a1, a2, lambda, L_v));
            W[(row - row_begin) * n3 + col] =
                wtN[l] * wtN[m] * wtN[n] * 0.25 * pow(0.5 * (d_i + d_j), 2) * g;
        }
    }
    free(wtN);
}

void oracle_weights_iso(int N, const double *zeta, double L_v, double lambda,
                        double d_i, double d_j, double m_i, double m_j,
                        int row_begin, int row_end, double *W, int nthreads)
{
    weights_iso_rows(N, zeta, L_v, lambda, d_i, d_j, m_i, m_j, row_begin, row_end, W,
                     nthreads, 0);
}

void oracle_weights_iso_closed(int N, const double *zeta, double L_v, double lambda,
                               double d_i, double d_j, double m_i, double m_j,
                               int row_begin, int row_end, double *W, int nthreads)
{
    weights_iso_rows(N, zeta, L_v, lambda, d_i, d_j, m_i, m_j, row_begin, row_end, W,
                     nthreads, 1);
}

/* -------------------------------------------------------------- 0D driver */
void oracle_init_bkw(int N, const double *v, double K, double *f)
{
    /* initializer.c:123-135 */
    double Temp = 1.0;
    if (!(K > 0)) K = 1 - exp(-5.5 / 6.0);
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                double v2 = v[i] * v[i] + v[j] * v[j] + v[k] * v[k];
                f[k + N * (j + N * i)] =
                    (exp(-(v2) / (2 * K * Temp * Temp))) / (2.0 * pow(2 * M_PI * K * Temp * Temp, 1.5)) *
                    ((5 * K - 3) / K + (1 - K) * (v2) / (K * K * Temp * Temp));
            }
}

static void stream_row(int N, const double *v, const double *f, double time,
                       double *row)
{
    /* write_streams, output.c:159-213 (mass 1, KB 1) */
    double bulkV[3], energy[2];
    double density = oracle_density(N, v, f, 1.0);
    oracle_bulk_velocity(N, v, f, density, 1.0, bulkV);
    double kinTemp = oracle_temperature(N, v, f, bulkV, density, 1.0, 1.0);
    oracle_energy(N, v, f, energy);
    row[0] = time;
    row[1] = density;
    row[2] = bulkV[0];
    row[3] = kinTemp;
    row[4] = density * kinTemp;
    row[5] = energy[1] / energy[0];
    for (int l = 0; l < N; l++) row[6 + l] = f[N / 2 + N * (N / 2 + N * l)];
}

void oracle_run_0d(int N, double L_v, const double *W, double *f, double dt,
                   double Kn, int nT, int order, int maxpreserve,
                   double *rows, int nthreads)
{
    /* boltz.c:186-250 for one species of mass 1 */
    long n3 = (long)N * N * N;
    double *v = (double *)malloc(sizeof(double) * N);
    double *zeta = (double *)malloc(sizeof(double) * N);
    oracle_grid_0d(N, L_v, v, zeta);
    double *Q = (double *)malloc(sizeof(double) * n3);
    double *f1 = (double *)malloc(sizeof(double) * n3);
    oracle_cons cons;
    double mass = 1.0;
    oracle_conservation_init(&cons, N, v[1] - v[0], v, &mass, 1);
    int stride = 6 + N;
    stream_row(N, v, f, 0.0, rows);
    for (int t = 0; t < nT; t++) {
        if (maxpreserve)
            oracle_computeQ_maxPreserve(N, L_v, v, zeta, W, f, f, Q, 1.0, 1.0, nthreads);
        else
            oracle_computeQ(N, L_v, v, zeta, W, f, f, Q, nthreads);
        oracle_conserve(&cons, &Q);
        if (order == 1) {
            for (long x = 0; x < n3; x++) f[x] += dt * Q[x] / Kn;
        } else {
            for (long x = 0; x < n3; x++) { f1[x] = f[x]; f1[x] += dt * Q[x] / Kn; }
            if (maxpreserve)
                oracle_computeQ_maxPreserve(N, L_v, v, zeta, W, f1, f1, Q, 1.0, 1.0, nthreads);
            else
                oracle_computeQ(N, L_v, v, zeta, W, f1, f1, Q, nthreads);
            oracle_conserve(&cons, &Q);
            for (long x = 0; x < n3; x++) {
                f[x] = 0.5 * (f[x] + f1[x]);
                f[x] += 0.5 * dt * Q[x] / Kn;
            }
        }
        stream_row(N, v, f, dt * (t + 1), rows + (long)(t + 1) * stride);
    }
    free(v); free(zeta); free(Q); free(f1);
}

/* ------------------------------------------------------------ 1D driver */
#define KB_JOULES 1.380658e-23 /* constants.h:6 */

void oracle_mesh_uniform(int nX, double length, int order, double *x, double *dx)
{
    /* mesh_setup.c:59-160 for one zone on one rank: x = cell centres */
    double dxz = length / (double)nX, x_edge = 0.0;
    for (int j = 0; j < nX; j++) {
        dx[order + j] = dxz;
        x[order + j] = x_edge + 0.5 * dxz;
        x_edge += dxz;
    }
    for (int g = order - 1; g >= 0; g--) {
        dx[g] = dx[g + 1];
        x[g] = x[g + 1] - dx[g + 1];
    }
    /* the reference leaves the right ghost cells unset on a single rank
       (the rank-0 branch of make_mesh); extend the grid uniformly */
    for (int g = nX + order; g < nX + 2 * order; g++) {
        dx[g] = dx[g - 1];
        x[g] = x[g - 1] + dx[g - 1];
    }
}

void oracle_init_1d(const oracle_1d *p, const double *v, double *f)
{
    /* initializer.c:296-424 */
    int N = p->N, nX = p->nX, order = p->order;
    long n3 = (long)N * N * N;
    double Ma = 1, TWall = 1.0;
    double rho_l = 1.0, ux_l = 0.0, T_l = 1.0, rho_r = 1.0, ux_r = 0.0, T_r = 1.0;
    double KB = p->KB, mass = p->mass;
    switch (p->ic) {
    case 0:
        rho_l = 4.0 * Ma * Ma / (Ma * Ma + 3.0);
        T_l = (5.0 * Ma * Ma - 1.0) * (Ma * Ma + 3.0) / (16.0 * Ma * Ma);
        ux_l = -sqrt(5.0 / 3.0) * (Ma * Ma + 3.0) / (4.0 * Ma);
        rho_r = 1.0; T_r = 1.0; ux_r = -Ma * sqrt(5.0 / 3.0);
        break;
    case 1: rho_r = 1.0; T_r = TWall; break;
    case 2: rho_l = 1.0; T_r = 2.0; T_l = 1.0; ux_l = -1.0; ux_r = -1.0; break;
    case 3: rho_r = 1.0; T_r = 1.5; break;
    case 5: rho_l = 1.0; T_l = 1.0; break;
    case 6: rho_l = 1.0; ux_l = 1.2972; T_l = 1.0; rho_r = 1.297; ux_r = 1.0; T_r = 1.195; break;
    }
    double maxTemp = T_r;
    for (int l = order; l < nX + order; l++) {
        double *fl = f + (long)l * n3;
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++)
                for (int k = 0; k < N; k++) {
                    long x = k + N * (j + (long)N * i);
                    double val = 0.0;
                    switch (p->ic) {
                    case 0:
                        if (l < nX / 2)
                            val = rho_l * exp(-((v[i]) * (v[i]) + v[j] * v[j] + v[k] * v[k]) / T_l) /
                                  ((T_l * M_PI) * sqrt(T_l * M_PI));
                        else
                            val = rho_r * exp(-((v[i]) * (v[i]) + v[j] * v[j] + v[k] * v[k]) / T_r) /
                                  ((T_r * M_PI) * sqrt(T_r * M_PI));
                        break;
                    case 1:
                        val = (rho_r / mass) * pow(0.5 * mass / (M_PI * KB * maxTemp), 1.5) *
                              exp(-(0.5 * mass / (KB * maxTemp)) * ((v[i]) * (v[i]) + v[j] * v[j] + v[k] * v[k]));
                        break;
                    case 2:
                        val = rho_l * exp(-((v[i] - ux_l) * (v[i] - ux_l) + v[j] * v[j] + v[k] * v[k]) / T_l) /
                              ((T_l * M_PI) * sqrt(T_l * M_PI));
                        break;
                    case 3:
                        val = rho_r * exp(-(v[i] * v[i] + v[j] * v[j] + v[k] * v[k]) / T_r) /
                              ((T_r * M_PI) * sqrt(T_r * M_PI));
                        break;
                    case 5:
                        val = rho_l * exp(-(v[i] * v[i] + v[j] * v[j] + v[k] * v[k]) / T_l) /
                              ((T_l * M_PI) * sqrt(T_l * M_PI));
                        break;
                    case 6:
                        if (l < nX / 2)
                            val = rho_l * exp(-((v[i] - ux_l) * (v[i] - ux_l) + v[j] * v[j] + v[k] * v[k]) / T_l) /
                                  ((T_l * M_PI) * sqrt(T_l * M_PI));
                        else
                            val = rho_r * exp(-((v[i] - ux_r) * (v[i] - ux_r) + v[j] * v[j] + v[k] * v[k]) / T_r) /
                                  ((T_r * M_PI) * sqrt(T_r * M_PI));
                        break;
                    }
                    fl[x] = val;
                }
    }
    (void)ux_r;
}

void oracle_diffuse_bc(int N, const double *v, const double *in, double *out,
                       double TW, int bdry, double mass, double KB)
{
    /* boundaryConditions.c:39-96 */
    double wtN[4096];
    trap_weights(N, wtN);
    double h_v = v[1] - v[0], sigmaW = 0.0;
    int ilo = bdry == 0 ? 0 : N / 2, ihi = bdry == 0 ? N / 2 : N;
    for (int i = ilo; i < ihi; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++)
                sigmaW += v[i] * wtN[i] * wtN[j] * wtN[k] * h_v * h_v * h_v * in[k + N * (j + N * i)];
    if (bdry == 0) sigmaW *= -sqrt(2.0 * M_PI * mass / (KB * TW));
    else sigmaW *= sqrt(2.0 * M_PI * mass / (KB * TW));
    int olo = bdry == 0 ? N / 2 : 0, ohi = bdry == 0 ? N : N / 2;
    for (int i = olo; i < ohi; i++)
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++)
                out[k + N * (j + N * i)] = sigmaW * pow(0.5 * mass / (M_PI * KB * TW), 1.5) *
                    exp(-0.5 * mass / (KB * TW) * (v[i] * v[i] + v[j] * v[j] + v[k] * v[k]));
}

static double mm_min(double a, double b) { return a > b ? b : a; }
static double mm_max(double a, double b) { return a > b ? a : b; }
static double minmod3(double a, double b, double c)
{
    /* transportroutines.c:80-90 */
    if ((a > 0) && (b > 0) && (c > 0)) return mm_min(mm_min(a, b), c);
    else if ((a < 0) && (b < 0) && (c < 0)) return mm_max(mm_max(a, b), c);
    return 0;
}

static void upwind_one(const oracle_1d *p, const double *v, double *f, double *fc)
{
    /* transportroutines.c:94-238 on one rank */
    int N = p->N, nX = p->nX, ic = p->ic;
    long n3 = (long)N * N * N;
    double *F0 = f, *F1 = f + n3, *Fn = f + (long)nX * n3, *Fn1 = f + (long)(nX + 1) * n3;
    if (ic == 3 || ic == 5) oracle_diffuse_bc(N, v, F1, F0, p->T0, 0, p->mass, p->KB);
    else if (ic == 1) oracle_diffuse_bc(N, v, F1, F0, 2.0 * p->TWall, 0, p->mass, p->KB);
    else if (ic != 6) memcpy(F0, F1, sizeof(double) * n3);
    if (ic == 3 || ic == 5) oracle_diffuse_bc(N, v, Fn, Fn1, p->T1, 1, p->mass, p->KB);
    else if (ic != 6) memcpy(Fn1, Fn, sizeof(double) * n3);
    if (ic == 6) {
        memcpy(F0, Fn, sizeof(double) * n3);
        memcpy(Fn1, F1, sizeof(double) * n3);
    }
    double Ma = 1.0;
    for (int l = 1; l < nX + 1; l++) {
        const double *fl = f + (long)l * n3, *fm = f + (long)(l - 1) * n3, *fp = f + (long)(l + 1) * n3;
        double *out = fc + (long)l * n3;
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) {
                for (int k = 0; k < N; k++) {
                    long x = k + N * (j + (long)N * i);
                    double CFL_NUM = p->dt * v[i] / p->dx[l];
                    if (i < N / 2) out[x] = (1.0 + CFL_NUM) * fl[x] - CFL_NUM * fp[x];
                    else out[x] = (1.0 - CFL_NUM) * fl[x] + CFL_NUM * fm[x];
                }
                if (ic == 5) {
                    for (int k = 0; k < N; k++) {
                        long x = k + N * (j + (long)N * i);
                        double c = Ma * p->dt / (2 * p->dx[l]);
                        if (j == 0) out[x] = out[x] - c * fl[k + N * ((j + 1) + N * i)];
                        else if (j == N - 1) out[x] = out[x] - c * fl[k + N * ((j - 1) + N * i)];
                        else out[x] = out[x] - c * (fl[k + N * ((j + 1) + N * i)] - fl[k + N * ((j - 1) + N * i)]);
                    }
                }
            }
    }
}

static void upwind_two(const oracle_1d *p, const double *v, double *f, double *fc,
                       double *f_l, double *f_r)
{
    /* transportroutines.c:241-470 on one rank */
    int N = p->N, nX = p->nX, ic = p->ic;
    long n3 = (long)N * N * N;
    const double *x = p->x, *dx = p->dx;
    double h_v = v[1] - v[0], Ma = 1.0;
#define FL(l) (f + (long)(l) * n3)
    for (long q = 0; q < n3; q++) {
        FL(1)[q] = 2 * FL(2)[q] - FL(3)[q];
        FL(nX + 2)[q] = 2 * FL(nX + 1)[q] - FL(nX)[q];
        /* cells 0 and nX+3 are not filled by the reference on one rank;
           their values only reach slopes that are never used */
        FL(0)[q] = FL(1)[q];
        FL(nX + 3)[q] = FL(nX + 2)[q];
    }
    for (int l = 2; l < nX + 2; l++) {
        if (l == 2) {
            for (int i = 0; i < N / 2; i++)
                for (int j = 0; j < N; j++)
                    for (int k = 0; k < N; k++) {
                        long q = k + N * (j + (long)N * i);
                        double s1 = minmod3((FL(2)[q] - FL(1)[q]) / (x[2] - x[1]),
                                            (FL(3)[q] - FL(2)[q]) / (x[3] - x[2]),
                                            (FL(3)[q] - FL(1)[q]) / (x[3] - x[1]));
                        f_l[q] = FL(2)[q] - 0.5 * dx[2] * s1;
                    }
            if (ic == 3 || ic == 5) oracle_diffuse_bc(N, v, f_l, f_l, p->T0, 0, p->mass, p->KB);
            else if (ic == 1) oracle_diffuse_bc(N, v, f_l, f_l, 2.0 * p->TWall, 0, p->mass, p->KB);
            else {
                for (int j = 0; j < N; j++)
                    for (int k = 0; k < N; k++)
                        for (int i = N / 2; i < N; i++) {
                            long q = k + N * (j + (long)N * i);
                            double s1 = minmod3((FL(2)[q] - FL(1)[q]) / (x[2] - x[1]),
                                                (FL(3)[q] - FL(2)[q]) / (x[3] - x[2]),
                                                (FL(3)[q] - FL(1)[q]) / (x[3] - x[1]));
                            f_l[q] = FL(2)[q] + 0.5 * dx[2] * s1;
                        }
            }
        }
        if (l == nX + 1) {
            for (int i = N / 2; i < N; i++)
                for (int j = 0; j < N; j++)
                    for (int k = 0; k < N; k++) {
                        long q = k + N * (j + (long)N * i);
                        double s1 = minmod3((FL(nX + 1)[q] - FL(nX)[q]) / (x[nX + 1] - x[nX]),
                                            (FL(nX + 2)[q] - FL(nX + 1)[q]) / (x[nX + 2] - x[nX + 1]),
                                            (FL(nX + 2)[q] - FL(nX)[q]) / (x[nX + 2] - x[nX]));
                        f_r[q] = FL(nX + 1)[q] + 0.5 * dx[nX + 1] * s1;
                    }
            if (ic == 3 || ic == 5) oracle_diffuse_bc(N, v, f_r, f_r, p->T1, l, p->mass, p->KB);
            else {
                for (int i = 0; i < N / 2; i++)
                    for (int j = 0; j < N; j++)
                        for (int k = 0; k < N; k++) {
                            long q = k + N * (j + (long)N * i);
                            double s1 = minmod3((FL(nX + 1)[q] - FL(nX)[q]) / (x[nX + 1] - x[nX]),
                                                (FL(nX + 2)[q] - FL(nX + 1)[q]) / (x[nX + 2] - x[nX + 1]),
                                                (FL(nX + 2)[q] - FL(nX)[q]) / (x[nX + 2] - x[nX]));
                            f_r[q] = FL(nX + 1)[q] - 0.5 * dx[nX + 1] * s1;
                        }
            }
        }
        double *out = fc + (long)l * n3;
        for (int j = 0; j < N; j++)
            for (int k = 0; k < N; k++) {
                for (int i = N / 2; i < N; i++) {
                    long q = k + N * (j + (long)N * i);
                    double s1 = minmod3((FL(l)[q] - FL(l - 1)[q]) / (x[l] - x[l - 1]),
                                        (FL(l + 1)[q] - FL(l)[q]) / (x[l + 1] - x[l]),
                                        (FL(l + 1)[q] - FL(l - 1)[q]) / (x[l + 1] - x[l - 1]));
                    double s0 = minmod3((FL(l - 1)[q] - FL(l - 2)[q]) / (x[l - 1] - x[l - 2]),
                                        (FL(l)[q] - FL(l - 1)[q]) / (x[l] - x[l - 1]),
                                        (FL(l)[q] - FL(l - 2)[q]) / (x[l] - x[l - 2]));
                    double CFL_NUM = 0.5 * p->dt * v[i] / dx[l];
                    if (l == 2)
                        out[q] = FL(l)[q] - CFL_NUM * (FL(l)[q] + 0.5 * dx[l] * s1 - f_l[q]);
                    else
                        out[q] = FL(l)[q] - CFL_NUM * (FL(l)[q] + 0.5 * dx[l] * s1 -
                                                      (FL(l - 1)[q] + 0.5 * dx[l - 1] * s0));
                    if (ic == 5) {
                        double c = Ma * 0.5 * p->dt / (2 * h_v);
                        if (j == 0) out[q] = out[q] - c * FL(l)[k + N * ((j + 1) + N * i)];
                        else if (j == N - 1) out[q] = out[q] - c * FL(l)[k + N * ((j - 1) + N * i)];
                        else out[q] = out[q] - c * (FL(l)[k + N * ((j + 1) + N * i)] - FL(l)[k + N * ((j - 1) + N * i)]);
                    }
                }
                for (int i = 0; i < N / 2; i++) {
                    long q = k + N * (j + (long)N * i);
                    double s2 = minmod3((FL(l + 1)[q] - FL(l)[q]) / (x[l + 1] - x[l]),
                                        (FL(l + 2)[q] - FL(l + 1)[q]) / (x[l + 2] - x[l + 1]),
                                        (FL(l + 2)[q] - FL(l)[q]) / (x[l + 2] - x[l]));
                    double s1 = minmod3((FL(l)[q] - FL(l - 1)[q]) / (x[l] - x[l - 1]),
                                        (FL(l + 1)[q] - FL(l)[q]) / (x[l + 1] - x[l]),
                                        (FL(l + 1)[q] - FL(l - 1)[q]) / (x[l + 1] - x[l - 1]));
                    double CFL_NUM = 0.5 * p->dt * v[i] / dx[l];
                    if (l == nX + 1)
                        out[q] = FL(l)[q] - CFL_NUM * (f_r[q] - (FL(l)[q] - 0.5 * dx[l] * s1));
                    else
                        out[q] = FL(l)[q] - CFL_NUM * (FL(l + 1)[q] - 0.5 * dx[l + 1] * s2 -
                                                      (FL(l)[q] - 0.5 * dx[l] * s1));
                    if (ic == 5) {
                        double c = Ma * 0.5 * p->dt / (2 * h_v);
                        if (j == 0) out[q] = out[q] - c * FL(l)[k + N * ((j + 1) + N * i)];
                        else if (j == N - 1) out[q] = out[q] - c * FL(l)[k + N * ((j - 1) + N * i)];
                        else out[q] = out[q] - c * (FL(l)[k + N * ((j + 1) + N * i)] - FL(l)[k + N * ((j - 1) + N * i)]);
                    }
                }
            }
    }
#undef FL
}

void oracle_advect(const oracle_1d *p, const double *v, double *f, double *fconv,
                   double *scratch)
{
    int N = p->N, nX = p->nX;
    long n3 = (long)N * N * N;
    if (p->order == 1) {
        upwind_one(p, v, f, fconv);
        return;
    }
    /* advectTwo, transportroutines.c:477-492; scratch = f_tmp + f_l + f_r */
    double *ftmp = scratch, *f_l = scratch + (long)(nX + 4) * n3, *f_r = f_l + n3;
    upwind_two(p, v, f, ftmp, f_l, f_r);
    upwind_two(p, v, ftmp, fconv, f_l, f_r);
    for (int l = 2; l < nX + 2; l++)
        for (long q = 0; q < n3; q++)
            fconv[(long)l * n3 + q] = 0.5 * (f[(long)l * n3 + q] + fconv[(long)l * n3 + q]);
}

static void stream_row_1d(const oracle_1d *p, const double *v, const double *f, double time,
                          double *rows)
{
    /* write_streams_inhom, output.c:295-340 */
    int N = p->N;
    long n3 = (long)N * N * N;
    for (int l = p->order; l < p->nX + p->order; l++) {
        double bulkV[3];
        const double *fl = f + (long)l * n3;
        double density = oracle_density(N, v, fl, p->mass);
        oracle_bulk_velocity(N, v, fl, density, p->mass, bulkV);
        double kinTemp = oracle_temperature(N, v, fl, bulkV, density, p->mass, p->KB);
        double *r = rows + (long)(l - p->order) * 6;
        r[0] = time; r[1] = p->x[l]; r[2] = density; r[3] = bulkV[0];
        r[4] = kinTemp; r[5] = density * kinTemp;
    }
}

void oracle_run_1d(const oracle_1d *p, const double *W, double *f, int nT,
                   double *rows, int nthreads)
{
    /* boltz.c:254-394 for one species on one rank */
    int N = p->N, nX = p->nX, order = p->order;
    long n3 = (long)N * N * N, ncell = nX + 2 * order;
    double *v = (double *)malloc(sizeof(double) * N);
    double *zeta = (double *)malloc(sizeof(double) * N);
    oracle_grid_1d(N, p->L_v, v, zeta);
    double *fconv = (double *)calloc((size_t)ncell * n3, sizeof(double));
    double *f1 = (double *)calloc((size_t)ncell * n3, sizeof(double));
    double *scratch = (double *)calloc((size_t)(nX + 6) * n3, sizeof(double));
    double *Q = (double *)malloc(sizeof(double) * n3);
    oracle_cons cons;
    double mass = p->mass;
    oracle_conservation_init(&cons, N, v[1] - v[0], v, &mass, 1);
    stream_row_1d(p, v, f, 0.0, rows);
    for (int t = 0; t < nT; t++) {
        oracle_advect(p, v, f, fconv, scratch);
        for (int l = order; l < nX + order; l++) {
            double *fc = fconv + (long)l * n3;
            oracle_computeQ(N, p->L_v, v, zeta, W, fc, fc, Q, nthreads);
            oracle_conserve(&cons, &Q);
            double *dst = (order == 1) ? f + (long)l * n3 : f1 + (long)l * n3;
            for (long q = 0; q < n3; q++) {
                dst[q] = fc[q];
                dst[q] += p->dt * Q[q] / p->Kn;
            }
            if (order == 2) {
                double *g1 = f1 + (long)l * n3;
                oracle_computeQ(N, p->L_v, v, zeta, W, g1, g1, Q, nthreads);
                oracle_conserve(&cons, &Q);
                for (long q = 0; q < n3; q++) {
                    fc[q] = 0.5 * fc[q] + 0.5 * g1[q];
                    fc[q] += 0.5 * p->dt * Q[q] / p->Kn;
                }
            }
        }
        if (order == 2) oracle_advect(p, v, fconv, f, scratch);
        stream_row_1d(p, v, f, p->dt * (t + 1), rows + (long)(t + 1) * nX * 6);
    }
    free(v); free(zeta); free(fconv); free(f1); free(scratch); free(Q);
}

/* gHat3L (aniso_weights.c:370-400): the Landau-kernel weight, a 64-point
   Gauss-Legendre rule in r on [0, L_v] around a 64-point rule in theta on
   [0, pi], as gsl_integration_glfixed applies it (nodes mid + half x_q,
   result half sum w_q f).  j0 is the C library's Bessel J0, as the
   reference calls it.  The operation order follows the reference. */
double oracle_ghat3l(double zeta1, double zeta2, double zeta3, double xi1, double xi2,
                     double xi3, double L_v, double lambda)
{
    static double gx[64], gw[64];
    static int init = 0;
    if (!init) {
#pragma omp critical(oracle_gl64)
        {
            if (!init) { oracle_gauss_legendre(64, gx, gw); init = 1; }
        }
    }
    double zetalen2 = zeta3 * zeta3 + zeta2 * zeta2 + zeta1 * zeta1;
    double xilen2 = xi1 * xi1 + xi2 * xi2 + xi3 * xi3;
    double xizeta = xi1 * zeta1 + xi2 * zeta2 + xi3 * zeta3;
    double zetalen = sqrt(zetalen2);
    double xiperp;
    if (((xilen2 - xizeta * xizeta / zetalen2) < 0) || (zetalen2 == 0))
        xiperp = 0;
    else
        xiperp = sqrt(xilen2 - xizeta * xizeta / zetalen2);
    double a0 = xiperp, a1 = zetalen2, a2 = zetalen != 0 ? xizeta / zetalen : 0.0, a3 = zetalen;
    double rmid = 0.5 * L_v, rhalf = 0.5 * L_v, tmid = 0.5 * M_PI, thalf = 0.5 * M_PI;
    double outer = 0.0;
    for (int p = 0; p < 64; p++) {
        double r = rmid + rhalf * gx[p], inner = 0.0;
        for (int q = 0; q < 64; q++) {
            double th = tmid + thalf * gx[q];
            double f = sin(th) * j0(r * a0 * sin(th)) *
                       (-r * r * a1 * sin(th) * sin(th) * cos(r * a2 * cos(th)) +
                        4 * r * a3 * sin(r * a2 * cos(th)) * cos(th));
            inner += gw[q] * f;
        }
        outer += gw[p] * (pow(r, lambda + 2) * (thalf * inner));
    }
    return 2.0 * M_PI * (rhalf * outer);
}

/* Rows [row0, row0 + nrows) of the Landau weights as
   generate_conv_weights_AnIso fills them (aniso_weights.c:402-425):
   W[z][n + N (m + N l)] = gHat3L(eta_i, eta_j, eta_k, eta_l, eta_m, eta_n). */
void oracle_weights_landau(int N, const double *eta, double L_v, double lambda, int row0,
                           int nrows, double *W)
{
    long n3 = (long)N * N * N;
#pragma omp parallel for schedule(dynamic)
    for (int zr = 0; zr < nrows; zr++) {
        int z = row0 + zr, k = z % N, j = ((z - k) / N) % N, i = (z - k - N * j) / (N * N);
        for (int l = 0; l < N; l++)
            for (int m = 0; m < N; m++)
                for (int n = 0; n < N; n++)
                    W[(long)zr * n3 + n + N * (m + (long)N * l)] =
                        oracle_ghat3l(eta[i], eta[j], eta[k], eta[l], eta[m], eta[n], L_v, lambda);
    }
}

/* ------------------------------------------------- grazing-collision weights
   gHat3 of the reference's stand-alone generator (MPIcollisionRoutines.c:
   33-205): for zeta and xi, with zl = |zeta|, xz = xi.zeta / zl and
   xp = |xi - xz zeta / zl| (both 0 when zl = 0),
     W = 4 pi^2 int_0^{L_v} r^{lambda+2} int_0^pi sin(phi) J0(r sin(phi) xp)
           [ I1(r, phi) + C(r, phi) (2/pi) log(g) / log(sin(g/2)) ] dphi dr
     I1 = int_{sqrt g}^{pi} (8/pi) (g / theta^2) theta^-2
            [cos(a7 (1 - cos theta) - a6) J0(a8 sin theta) - cos(a6)] dtheta
     a6 = r cos(phi) xz, a7 = r cos(phi) zl / 2, a8 = r sin(phi) zl / 2,
     C  = -a8^2 cos(a6) / 4 + a7 sin(a6) / 2
   (:33-52 ghat_theta, :83-121 ghat_phi with the Coulomb-case Taylor term of
   :112-119, :124-143 ghat_r, :154-205 gHat3).  The reference integrates with
   GSL QAG (61 points, 1e-6) in r and phi and CQUAD (1e-6) in theta.  Here
   every level is composite 16-point Gauss-Legendre, converged to ~1e-13:
   npan equal panels in r and in phi, and in theta panels graded
   geometrically from sqrt(g) by a factor 2 (the integrand grows like
   theta^-2 towards sqrt(g)).  Parity with GSL's 1e-6 answers is not pinned:
   no GSL CQUAD exists here. */
int oracle_graze_theta_edges(double glance, double *edges /* >= 64 */)
{
    int n = 0;
    double t = sqrt(glance);
    edges[n++] = t;
    while (2.0 * t < M_PI && n < 62) {
        t *= 2.0;
        edges[n++] = t;
    }
    edges[n++] = M_PI;
    return n - 1; /* panels */
}

int oracle_graze_panels(double L_eta, double L_v)
{
    /* the integrands' phase in r and phi stays below |zeta| + |xi| <=
       2 sqrt(3) L_eta per unit r; 16-point panels spanning <= 8 rad of it */
    int K = (int)ceil(2.0 * sqrt(3.0) * L_eta * L_v / 8.0);
    return K < 2 ? 2 : K;
}

double oracle_ghat3_graze(double zeta1, double zeta2, double zeta3, double xi1, double xi2,
                          double xi3, double L_v, double lambda, double glance, int npan)
{
    static double gx[16], gw[16];
    static int init = 0;
    if (!init) {
#pragma omp critical(oracle_gl16)
        {
            if (!init) { oracle_gauss_legendre(16, gx, gw); init = 1; }
        }
    }
    double zetalen2 = zeta1 * zeta1 + zeta2 * zeta2 + zeta3 * zeta3;
    double xilen2 = xi1 * xi1 + xi2 * xi2 + xi3 * xi3;
    double xizeta = xi1 * zeta1 + xi2 * zeta2 + xi3 * zeta3;
    double zl = sqrt(zetalen2), xp;
    if (((xilen2 - xizeta * xizeta / zetalen2) < 0) || (zetalen2 == 0))
        xp = 0;
    else
        xp = sqrt(xilen2 - xizeta * xizeta / zetalen2);
    double xz = zl != 0 ? xizeta / zl : 0.0;
    double te[64];
    int nte = oracle_graze_theta_edges(glance, te);
    double taylor = (2.0 / M_PI) * log(glance) / log(sin(0.5 * glance));
    double hr = L_v / npan, hp = M_PI / npan;
    double total = 0.0;
    for (int pr = 0; pr < npan; pr++)
        for (int qr = 0; qr < 16; qr++) {
            double r = hr * pr + 0.5 * hr * (gx[qr] + 1.0);
            double phisum = 0.0;
            for (int pp = 0; pp < npan; pp++)
                for (int qp = 0; qp < 16; qp++) {
                    double phi = hp * pp + 0.5 * hp * (gx[qp] + 1.0);
                    double cph = cos(phi), sph = sin(phi);
                    double a6 = r * cph * xz, a7 = 0.5 * r * cph * zl, a8 = 0.5 * r * sph * zl;
                    double a9 = cos(a6);
                    double i1 = 0.0;
                    for (int pt = 0; pt < nte; pt++) {
                        double t0 = te[pt], ht = te[pt + 1] - te[pt], s = 0.0;
                        for (int qt = 0; qt < 16; qt++) {
                            double th = t0 + 0.5 * ht * (gx[qt] + 1.0);
                            double bcos = (8.0 / M_PI) * (glance / (th * th)) / (th * th);
                            s += gw[qt] * bcos *
                                 (cos(a7 * (1.0 - cos(th)) - a6) * j0(a8 * sin(th)) - a9);
                        }
                        i1 += 0.5 * ht * s;
                    }
                    double C = -0.25 * a8 * a8 * cos(a6) + 0.5 * a7 * sin(a6);
                    phisum += 0.5 * hp * gw[qp] * sph * j0(r * sph * xp) * (i1 + C * taylor);
                }
            total += 0.5 * hr * gw[qr] * pow(r, lambda + 2) * phisum;
        }
    return 4.0 * M_PI * M_PI * total;
}

/* gHat3 of the grazing generator for npairs (zeta, xi) pairs, pairs[6 p ..
   6 p + 5] = zeta1..3, xi1..3, OpenMP over pairs. */
void oracle_ghat3_graze_pairs(int npairs, const double *pairs, double L_v, double lambda,
                              double glance, int npan, double *out)
{
#pragma omp parallel for schedule(dynamic)
    for (int p = 0; p < npairs; p++) {
        const double *q = pairs + 6L * p;
        out[p] = oracle_ghat3_graze(q[0], q[1], q[2], q[3], q[4], q[5], L_v, lambda, glance,
                                    npan);
    }
}
