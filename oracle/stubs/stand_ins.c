/*
 * stand_ins.c -- project-written implementations of the FFTW, GSL and MPI
 * entry points that the reference's sources call.  With them, those
 * sources build into the CPU reference under oracle/_ref.
 * TEST INFRASTRUCTURE.  Nothing from the libraries is copied: each function
 * does what its documented interface promises, restated in plain C.
 */
#include "fftw3.h"
#include "mpi.h"
#include "gsl/gsl_integration.h"
#include "../dft3.h"
#include "../spectral_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

/* ---------------------------------------------------------------- FFTW */
struct oracle_fftw_plan_s {
    int n0, n1, n2, sign;
    double *in, *out;
};

void *fftw_malloc(size_t n) { return malloc(n); }
void fftw_free(void *p) { free(p); }

fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags)
{
    (void)flags;
    fftw_plan p = (fftw_plan)malloc(sizeof(*p));
    p->n0 = n0; p->n1 = n1; p->n2 = n2; p->sign = sign;
    p->in = (double *)in; p->out = (double *)out;
    return p;
}

void fftw_execute(const fftw_plan p)
{
    size_t n = (size_t)p->n0 * p->n1 * p->n2;
    if (p->in != p->out) memcpy(p->out, p->in, sizeof(double) * 2 * n);
    oracle_dft3(p->n0, p->n1, p->n2, p->out, p->sign);
}

void fftw_destroy_plan(fftw_plan p) { free(p); }

/* ----------------------------------------------------------------- MPI */
int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }
double MPI_Wtime(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm c)
{
    (void)buf; (void)count; (void)t; (void)root; (void)c;
    return 0;
}
int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c)
{
    (void)buf; (void)count; (void)t; (void)tag; (void)c;
    fprintf(stderr, "single-rank MPI stand-in: MPI_Send to %d\n", dest);
    abort();
}
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st)
{
    (void)buf; (void)count; (void)t; (void)tag; (void)c; (void)st;
    fprintf(stderr, "single-rank MPI stand-in: MPI_Recv from %d\n", src);
    abort();
}
int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count)
{
    (void)t;
    *count = st ? st->count : 0;
    return 0;
}

/* ----------------------------------------------------------------- GSL */
#define QAG_PANELS 64
#define QAG_POINTS 16

gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n)
{
    gsl_integration_workspace *w = (gsl_integration_workspace *)malloc(sizeof(*w));
    w->limit = n;
    return w;
}
void gsl_integration_workspace_free(gsl_integration_workspace *w) { free(w); }

int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs,
                        double epsrel, size_t limit, int key,
                        gsl_integration_workspace *w, double *result, double *abserr)
{
    (void)epsabs; (void)epsrel; (void)limit; (void)key; (void)w;
    double x[QAG_POINTS], wt[QAG_POINTS];
    oracle_gauss_legendre(QAG_POINTS, x, wt);
    double h = (b - a) / QAG_PANELS, total = 0.0;
    for (int p = 0; p < QAG_PANELS; p++) {
        double mid = a + (p + 0.5) * h, part = 0.0;
        for (int q = 0; q < QAG_POINTS; q++)
            part += wt[q] * f->function(mid + 0.5 * h * x[q], f->params);
        total += 0.5 * h * part;
    }
    *result = total;
    if (abserr) *abserr = 0.0;
    return 0;
}

gsl_integration_cquad_workspace *gsl_integration_cquad_workspace_alloc(size_t n)
{
    gsl_integration_cquad_workspace *w = (gsl_integration_cquad_workspace *)malloc(sizeof(*w));
    w->n = n;
    return w;
}
void gsl_integration_cquad_workspace_free(gsl_integration_cquad_workspace *w) { free(w); }
int gsl_integration_cquad(const gsl_function *f, double a, double b, double epsabs,
                          double epsrel, gsl_integration_cquad_workspace *ws,
                          double *result, double *abserr, size_t *nevals)
{
    (void)f; (void)a; (void)b; (void)epsabs; (void)epsrel; (void)ws;
    (void)result; (void)abserr; (void)nevals;
    fprintf(stderr, "cquad is not available in the CPU reference build\n");
    abort();
}

gsl_integration_glfixed_table *gsl_integration_glfixed_table_alloc(size_t n)
{
    gsl_integration_glfixed_table *t = (gsl_integration_glfixed_table *)malloc(sizeof(*t));
    t->n = n;
    t->x = (double *)malloc(sizeof(double) * n);
    t->w = (double *)malloc(sizeof(double) * n);
    oracle_gauss_legendre((int)n, t->x, t->w);
    return t;
}
void gsl_integration_glfixed_table_free(gsl_integration_glfixed_table *t)
{
    free(t->x); free(t->w); free(t);
}
double gsl_integration_glfixed(const gsl_function *f, double a, double b,
                               const gsl_integration_glfixed_table *t)
{
    double mid = 0.5 * (a + b), half = 0.5 * (b - a), s = 0.0;
    for (size_t q = 0; q < t->n; q++) s += t->w[q] * f->function(mid + half * t->x[q], f->params);
    return half * s;
}
