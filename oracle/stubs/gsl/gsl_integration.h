/*
 * gsl_integration.h stand-in for building the reference under oracle/_ref.
 * TEST INFRASTRUCTURE.  GSL is absent from this image.
 *
 * gsl_integration_qag (weights.c:203) becomes composite Gauss-Legendre: 64
 * panels of 16 nodes, converged to round-off for the isotropic integrand.
 * The reference calls adaptive Gauss-Kronrod to 1e-8, so the weights agree
 * with the shipped .wts fixtures to about 1e-16 relative, not bit for bit.
 * glfixed is an n-point Gauss-Legendre rule.  cquad (the Coulomb path of
 * aniso_weights.c) aborts; that path is unsupported here.
 */
#ifndef ORACLE_STUB_GSL_INTEGRATION_H
#define ORACLE_STUB_GSL_INTEGRATION_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { double (*function)(double x, void *params); void *params; } gsl_function;
typedef struct { size_t limit; } gsl_integration_workspace;
typedef struct { size_t n; } gsl_integration_cquad_workspace;
typedef struct { size_t n; double *x; double *w; } gsl_integration_glfixed_table;
gsl_integration_workspace *gsl_integration_workspace_alloc(size_t n);
void gsl_integration_workspace_free(gsl_integration_workspace *w);
int gsl_integration_qag(const gsl_function *f, double a, double b, double epsabs,
                        double epsrel, size_t limit, int key,
                        gsl_integration_workspace *w, double *result, double *abserr);
gsl_integration_cquad_workspace *gsl_integration_cquad_workspace_alloc(size_t n);
void gsl_integration_cquad_workspace_free(gsl_integration_cquad_workspace *w);
int gsl_integration_cquad(const gsl_function *f, double a, double b, double epsabs,
                          double epsrel, gsl_integration_cquad_workspace *ws,
                          double *result, double *abserr, size_t *nevals);
gsl_integration_glfixed_table *gsl_integration_glfixed_table_alloc(size_t n);
void gsl_integration_glfixed_table_free(gsl_integration_glfixed_table *t);
double gsl_integration_glfixed(const gsl_function *f, double a, double b,
                               const gsl_integration_glfixed_table *t);
#ifdef __cplusplus
}
#endif
#endif
