// brent.cuh -- brent_find_root (src/math/root_finding.hpp:145-302) as a
// per-thread state machine that consumes one function value at a time, so
// that a caller can evaluate the objective however it likes (a batch of PDE
// marches for FDM IV, a surface lookup for interpolated IV).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace mgpu {

// Result codes of the root finders.
constexpr int32_t kIvOk = 0, kIvBracket = 1, kIvMaxIter = 2, kIvNumerical = 3;

// Brent state of one quote (root_finding.hpp:145-302 variables).
struct BrentDev {
  double a, b, c, d, fa, fb, fc, s;
  double root, ferr;
  int32_t iter, mflag, phase, code;  // phase: 0 eval a, 1 eval b, 2 eval s
};

namespace brentdev {

__device__ __forceinline__ void swap_d(double& x, double& y) {
  const double t = x;
  x = y;
  y = t;
}

__device__ __forceinline__ double qnan() { return __longlong_as_double(0x7ff8000000000000ll); }
__device__ __forceinline__ double pinf() { return __longlong_as_double(0x7ff0000000000000ll); }

// Convergence test and next trial point at the top of a Brent iteration;
// returns false when the quote is finished.
__device__ __forceinline__ bool brent_propose(BrentDev& s, double tol, int max_iter) {
  if (s.iter >= max_iter) {
    s.code = kIvMaxIter;
    s.root = s.b;
    s.ferr = fabs(s.fb);
    return false;
  }
  if (fabs(s.fb) < tol || fabs(s.b - s.a) < tol) {
    s.code = kIvOk;
    s.root = s.b;
    s.ferr = fabs(s.fb);
    s.iter += 1;  // the reference reports iter + 1 here
    return false;
  }
  const double a = s.a, b = s.b, c = s.c, fa = s.fa, fb = s.fb, fc = s.fc;
  double x;
  if (fa != fc && fb != fc) {  // inverse quadratic interpolation
    x = a * fb * fc / ((fa - fb) * (fa - fc)) + b * fa * fc / ((fb - fa) * (fb - fc)) +
        c * fa * fb / ((fc - fa) * (fc - fb));
  } else {  // secant
    x = b - fb * (b - a) / (fb - fa);
  }
  const double bis = (3.0 * a + b) / 4.0;
  const bool c1 = !((x > bis && x < b) || (x < bis && x > b));
  const bool c2 = s.mflag && fabs(x - b) >= fabs(b - c) / 2.0;
  const bool c3 = !s.mflag && fabs(x - b) >= fabs(c - s.d) / 2.0;
  const bool c4 = s.mflag && fabs(b - c) < tol;
  const bool c5 = !s.mflag && fabs(c - s.d) < tol;
  if (c1 || c2 || c3 || c4 || c5) {
    x = (a + b) / 2.0;
    s.mflag = 1;
  } else {
    s.mflag = 0;
  }
  s.s = x;
  return true;
}

__device__ __forceinline__ void brent_start(BrentDev& s, double lower, double upper) {
  s = BrentDev{};
  s.a = lower;
  s.b = upper;
  s.phase = 0;
  s.code = kIvNumerical;
}

// Consume the objective value f at the last trial point and advance Brent
// by one function value; returns true with the next trial point in *next,
// false when the quote is finished (code, root, ferr, iter set).
__device__ __forceinline__ bool brent_consume(BrentDev& s, double f, double tol, int max_iter, double* next) {
  if (s.phase == 0) {
    s.fa = f;
    s.phase = 1;
    *next = s.b;
    return true;
  }
  if (s.phase == 1) {
    s.fb = f;
    s.iter = 0;
    if (!isfinite(s.fa) || !isfinite(s.fb)) {
      s.code = kIvNumerical;
      s.ferr = qnan();
      return false;
    }
    if (s.fa * s.fb > 0.0) {
      s.code = kIvBracket;
      s.ferr = fmin(fabs(s.fa), fabs(s.fb));
      return false;
    }
    if (fabs(s.fa) < tol) {
      s.code = kIvOk;
      s.root = s.a;
      s.ferr = fabs(s.fa);
      return false;
    }
    if (fabs(s.fb) < tol) {
      s.code = kIvOk;
      s.root = s.b;
      s.ferr = fabs(s.fb);
      return false;
    }
    if (fabs(s.fa) < fabs(s.fb)) {
      swap_d(s.a, s.b);
      swap_d(s.fa, s.fb);
    }
    s.c = s.a;
    s.fc = s.fa;
    s.mflag = 1;
    s.d = 0.0;
    s.phase = 2;
    const bool go = brent_propose(s, tol, max_iter);
    *next = s.s;
    return go;
  }
  if (!isfinite(f)) {
    s.code = kIvNumerical;
    s.root = s.s;
    s.ferr = qnan();
    s.iter += 1;
    return false;
  }
  s.d = s.c;
  s.c = s.b;
  s.fc = s.fb;
  if (s.fa * f < 0.0) {
    s.b = s.s;
    s.fb = f;
  } else {
    s.a = s.s;
    s.fa = f;
  }
  if (fabs(s.fa) < fabs(s.fb)) {
    swap_d(s.a, s.b);
    swap_d(s.fa, s.fb);
  }
  s.iter += 1;
  const bool go = brent_propose(s, tol, max_iter);
  *next = s.s;
  return go;
}

}  // namespace brentdev
}  // namespace mgpu
