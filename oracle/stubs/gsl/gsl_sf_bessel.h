/* gsl_sf_bessel.h stand-in (TEST INFRASTRUCTURE): weights.c includes it but
   calls nothing from it; aniso_weights.c uses libm's j0. */
#ifndef ORACLE_STUB_GSL_SF_BESSEL_H
#define ORACLE_STUB_GSL_SF_BESSEL_H
#endif
