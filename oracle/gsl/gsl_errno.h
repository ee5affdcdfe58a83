/* GSL-API adapter for building the reference with the oracle's restated
 * special functions (oracle/specfun.c). TEST INFRASTRUCTURE ONLY. */
#ifndef PF_ORACLE_GSL_ERRNO_H
#define PF_ORACLE_GSL_ERRNO_H
#define GSL_SUCCESS 0
#define GSL_EDOM 1
#define GSL_EUNDRFLW 15
#define GSL_EOVRFLW 16
#endif
