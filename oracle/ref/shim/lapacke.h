/* Oracle build shim (test infrastructure only): LAPACKE is not installed
 * here.  The reference's collocation fit calls three banded routines; these
 * declarations let it compile, and lapacke_stubs.c forwards the calls to the
 * library MANGO_REF_LAPACKE names (or fails loudly without one). */
#pragma once
#include <stdint.h>
typedef int32_t lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
#ifdef __cplusplus
extern "C" {
#endif
lapack_int LAPACKE_dgbtrf(int layout, lapack_int m, lapack_int n, lapack_int kl, lapack_int ku,
                          double* ab, lapack_int ldab, lapack_int* ipiv);
lapack_int LAPACKE_dgbtrs(int layout, char trans, lapack_int n, lapack_int kl, lapack_int ku,
                          lapack_int nrhs, const double* ab, lapack_int ldab,
                          const lapack_int* ipiv, double* b, lapack_int ldb);
lapack_int LAPACKE_dgbcon(int layout, char norm, lapack_int n, lapack_int kl, lapack_int ku,
                          const double* ab, lapack_int ldab, const lapack_int* ipiv,
                          double anorm, double* rcond);
#ifdef __cplusplus
}
#endif
