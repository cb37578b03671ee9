/*
 * dft3.c -- direct separable 3D DFT (see dft3.h).  TEST INFRASTRUCTURE.
 */
#include "dft3.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* Transform `count` strided lines of length n in place.  Line l starts at
   element base(l) and its elements are `stride` apart. */
static void dft_lines(int n, int sign, double *data, long nlines_outer,
                      long outer_stride, long nlines_inner, long stride)
{
    double *cw = (double *)malloc(sizeof(double) * (size_t)n);
    double *sw = (double *)malloc(sizeof(double) * (size_t)n);
    double *tmp = (double *)malloc(sizeof(double) * 2 * (size_t)n);
    for (int m = 0; m < n; m++) {
        double a = 2.0 * M_PI * (double)m / (double)n;
        cw[m] = cos(a);
        sw[m] = (double)sign * sin(a);
    }
    for (long o = 0; o < nlines_outer; o++) {
        for (long in = 0; in < nlines_inner; in++) {
            double *line = data + 2 * (o * outer_stride + in);
            for (int k = 0; k < n; k++) {
                double re = 0.0, im = 0.0;
                for (int j = 0; j < n; j++) {
                    int m = (int)(((long)j * k) % n);
                    double xr = line[2 * (long)j * stride];
                    double xi = line[2 * (long)j * stride + 1];
                    re += xr * cw[m] - xi * sw[m];
                    im += xr * sw[m] + xi * cw[m];
                }
                tmp[2 * k] = re;
                tmp[2 * k + 1] = im;
            }
            for (int k = 0; k < n; k++) {
                line[2 * (long)k * stride] = tmp[2 * k];
                line[2 * (long)k * stride + 1] = tmp[2 * k + 1];
            }
        }
    }
    free(cw);
    free(sw);
    free(tmp);
}

void oracle_dft3(int n0, int n1, int n2, double *data, int sign)
{
    long s0 = (long)n1 * n2; /* stride of axis 0 */
    /* axis 2 (contiguous): n0*n1 lines */
    dft_lines(n2, sign, data, (long)n0 * n1, n2, 1, 1);
    /* axis 1: for each i0, n2 lines with stride n2 */
    dft_lines(n1, sign, data, n0, s0, n2, n2);
    /* axis 0: n1*n2 lines with stride s0 */
    dft_lines(n0, sign, data, 1, 0, s0, s0);
}
