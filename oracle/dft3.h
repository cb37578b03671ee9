/*
 * dft3.h -- unnormalised 3D complex discrete Fourier transform on the CPU.
 *
 * TEST INFRASTRUCTURE: part of the CPU oracle.  Only the tests, the smoke
 * check and bench.py's CPU-baseline leg use it.  It is never part of the
 * product path.
 *
 * Convention (the one the reference gets from FFTW through
 * fftw_plan_dft_3d, collisions.c:67-68):
 *   sign = -1 : X[k] = sum_n x[n] exp(-2 pi i n.k / N)   (FFTW_FORWARD)
 *   sign = +1 : X[k] = sum_n x[n] exp(+2 pi i n.k / N)   (FFTW_BACKWARD)
 * Neither direction scales.  The array is row major, the last index is
 * contiguous, and elements are interleaved (re, im) pairs like fftw_complex.
 *
 * The transform is separable.  A direct DFT runs along each axis with
 * exactly reduced twiddles, exp(+-2 pi i ((n k) mod N) / N), so any N
 * works, including the N=24 and odd-N grids the reference accepts.
 */
#ifndef ORACLE_DFT3_H
#define ORACLE_DFT3_H

#ifdef __cplusplus
extern "C" {
#endif

/* In-place 3D DFT of a (n0, n1, n2) interleaved complex array. */
void oracle_dft3(int n0, int n1, int n2, double *data, int sign);

#ifdef __cplusplus
}
#endif

#endif
