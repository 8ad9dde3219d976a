/* Test infrastructure only: see shim/lapacke.h.  Any call is an error. */
#include <stdio.h>
#include <stdlib.h>
#include "shim/lapacke.h"
static lapack_int fail(const char* f) {
  fprintf(stderr, "oracle reference build: %s is not available (no LAPACKE here)\n", f);
  return -1;
}
lapack_int LAPACKE_dgbtrf(int a, lapack_int b, lapack_int c, lapack_int d, lapack_int e, double* f,
                          lapack_int g, lapack_int* h) {
  (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h;
  return fail("LAPACKE_dgbtrf");
}
lapack_int LAPACKE_dgbtrs(int a, char b, lapack_int c, lapack_int d, lapack_int e, lapack_int f,
                          const double* g, lapack_int h, const lapack_int* i, double* j, lapack_int k) {
  (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j; (void)k;
  return fail("LAPACKE_dgbtrs");
}
lapack_int LAPACKE_dgbcon(int a, char b, lapack_int c, lapack_int d, lapack_int e, const double* f,
                          lapack_int g, const lapack_int* h, double i, double* j) {
  (void)a; (void)b; (void)c; (void)d; (void)e; (void)f; (void)g; (void)h; (void)i; (void)j;
  return fail("LAPACKE_dgbcon");
}
