/*
 * fftw3.h stand-in for compiling the reference's own sources into the CPU
 * reference build under oracle/_ref.  TEST INFRASTRUCTURE.
 *
 * FFTW3 is absent from this image.  This header declares the few FFTW
 * entry points that collisions.c uses (collisions.c:59-68, 82-87, 270).
 * stand_ins.c implements them with the direct DFT of dft3.c, using FFTW's
 * sign convention and no scaling.
 */
#ifndef ORACLE_STUB_FFTW3_H
#define ORACLE_STUB_FFTW3_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s *fftw_plan;
#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)
void *fftw_malloc(size_t n);
void fftw_free(void *p);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex *in,
                           fftw_complex *out, int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_destroy_plan(fftw_plan p);
#ifdef __cplusplus
}
#endif
#endif
