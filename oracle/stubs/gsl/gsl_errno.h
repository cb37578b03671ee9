/* gsl_errno.h stand-in (TEST INFRASTRUCTURE): nothing the reference uses. */
#ifndef ORACLE_STUB_GSL_ERRNO_H
#define ORACLE_STUB_GSL_ERRNO_H
#define GSL_SUCCESS 0
#endif
