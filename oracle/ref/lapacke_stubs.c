/* Test infrastructure only: see shim/lapacke.h.  LAPACKE is not installed
 * here.  When MANGO_REF_LAPACKE names a shared library that exports the
 * LAPACKE banded routines (plain, or with a "scipy_" prefix as in the
 * OpenBLAS that scipy bundles), the three calls of the reference's
 * collocation fit are forwarded to it, so that the reference's own fit runs
 * for the golden generator; otherwise every call fails loudly. */
#include <dlfcn.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include "shim/lapacke.h"

static void* lib = NULL;
static pthread_once_t once = PTHREAD_ONCE_INIT;
static void open_lib(void) {  /* once, whichever thread calls first */
  const char* path = getenv("MANGO_REF_LAPACKE");
  if (path && *path) lib = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (path && *path && !lib) fprintf(stderr, "oracle reference build: %s\n", dlerror());
}

static void* sym(const char* name) {
  pthread_once(&once, open_lib);
  if (!lib) return NULL;
  char prefixed[64];
  snprintf(prefixed, sizeof prefixed, "scipy_%s", name);
  void* f = dlsym(lib, prefixed);
  return f ? f : dlsym(lib, name);
}

static lapack_int fail(const char* f) {
  fprintf(stderr, "oracle reference build: %s is not available (set MANGO_REF_LAPACKE)\n", f);
  return -1;
}

typedef lapack_int (*dgbtrf_t)(int, lapack_int, lapack_int, lapack_int, lapack_int, double*,
                               lapack_int, lapack_int*);
typedef lapack_int (*dgbtrs_t)(int, char, lapack_int, lapack_int, lapack_int, lapack_int,
                               const double*, lapack_int, const lapack_int*, double*, lapack_int);
typedef lapack_int (*dgbcon_t)(int, char, lapack_int, lapack_int, lapack_int, const double*,
                               lapack_int, const lapack_int*, double, double*);

lapack_int LAPACKE_dgbtrf(int layout, lapack_int m, lapack_int n, lapack_int kl, lapack_int ku,
                          double* ab, lapack_int ldab, lapack_int* ipiv) {
  dgbtrf_t f = (dgbtrf_t)sym("LAPACKE_dgbtrf");
  return f ? f(layout, m, n, kl, ku, ab, ldab, ipiv) : fail("LAPACKE_dgbtrf");
}
lapack_int LAPACKE_dgbtrs(int layout, char trans, lapack_int n, lapack_int kl, lapack_int ku,
                          lapack_int nrhs, const double* ab, lapack_int ldab,
                          const lapack_int* ipiv, double* b, lapack_int ldb) {
  dgbtrs_t f = (dgbtrs_t)sym("LAPACKE_dgbtrs");
  return f ? f(layout, trans, n, kl, ku, nrhs, ab, ldab, ipiv, b, ldb) : fail("LAPACKE_dgbtrs");
}
lapack_int LAPACKE_dgbcon(int layout, char norm, lapack_int n, lapack_int kl, lapack_int ku,
                          const double* ab, lapack_int ldab, const lapack_int* ipiv,
                          double anorm, double* rcond) {
  dgbcon_t f = (dgbcon_t)sym("LAPACKE_dgbcon");
  return f ? f(layout, norm, n, kl, ku, ab, ldab, ipiv, anorm, rcond) : fail("LAPACKE_dgbcon");
}
