// march_dev.cuh -- device helpers shared by the march kernels: the
// projection max, the natural cubic spline and stencil read-outs, and
// AmericanOptionResult's functionals (src/option/american_option_result.cpp:
// 25-121) on a solved tile row.
#pragma once
#include "march.cuh"

namespace mgpu {
namespace {


// std::max(v, psi) for psi >= +0 (a payoff), with integer compares instead of
// an FP64 instruction: non-negative doubles order like their bit patterns and
// any negative v (sign bit set) loses.  Differs from the reference only for
// v = -0, psi = +0 (returns +0 instead of -0, the same number).
__device__ __forceinline__ double proj_max(double v, double psi) {
  const long long vb = __double_as_longlong(v), pb = __double_as_longlong(psi);
  return __longlong_as_double(vb > pb ? vb : pb);
}

__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b);
}




// Natural cubic spline through (x, y) (cubic_spline_solver.hpp:74-170,
// 264-369): solve for the second-derivative terms c_i with the plain Thomas
// recurrence (thomas_solver.hpp:86-198), then evaluate at xe on interval iv.
// The lane's A_CP / A_D rows serve as the c' / d' scratch.
// Thomas scratch of one evaluation: c'_j at cp[j * stride], d'_j at dp[j * stride].
struct SplineScratch {
  double* cp;
  double* dp;
  size_t stride;
  __device__ __forceinline__ double& C(int j) const { return cp[static_cast<size_t>(j) * stride]; }
  __device__ __forceinline__ double& D(int j) const { return dp[static_cast<size_t>(j) * stride]; }
};

template <class Y>
__device__ __forceinline__ void spline_eval(const double* __restrict__ X, Y y, int n, double xe,
                                            int iv, const SplineScratch& W, double* val,
                                            double* der) {
  auto x = [&](int i) { return ROW(X, i); };
  auto h = [&](int i) { return x(i + 1) - x(i); };
  double ci = 0.0, ci1 = 0.0;  // c[iv], c[iv+1]
  const int m = n - 2;
  if (m >= 1) {
    // system row j (0..m-1) for knot k = j+1:
    //   lower h[j] (j>0), diag 2(h[j]+h[j+1]), upper h[j+1] (j<m-1)
    auto rhs = [&](int j) {
      const double sr = (y(j + 2) - y(j + 1)) / h(j + 1);
      const double sl = (y(j + 1) - y(j)) / h(j);
      return 3.0 * (sr - sl);
    };
    if (m == 1) {
      const double s = rhs(0) / (2.0 * (h(0) + h(1)));
      if (iv == 0) {
        ci = 0.0;
        ci1 = s;
      } else {
        ci = s;
        ci1 = 0.0;
      }
    } else {
      const double diag0 = 2.0 * (h(0) + h(1));
      double cp = h(1) / diag0;
      double dp = rhs(0) / diag0;
      W.C(0) = cp;
      W.D(0) = dp;
      for (int j = 1; j < m - 1; ++j) {
        const double lower = h(j);
        const double denom = fma(-lower, cp, 2.0 * (h(j) + h(j + 1)));
        const double inv = 1.0 / denom;
        cp = h(j + 1) * inv;
        dp = fma(-lower, dp, rhs(j)) * inv;
        W.C(j) = cp;
        W.D(j) = dp;
      }
      {
        const int j = m - 1;
        const double lower = h(j);
        const double denom = fma(-lower, cp, 2.0 * (h(j) + h(j + 1)));
        dp = fma(-lower, dp, rhs(j)) / denom;
        W.D(j) = dp;
      }
      // back substitution: sol[j] = c[j+1]; only c[iv], c[iv+1] are needed.
      double s = W.D(m - 1);
      auto take = [&](int kk, double v) {
        if (kk == iv) ci = v;
        if (kk == iv + 1) ci1 = v;
      };
      take(m, s);
      for (int j = m - 1; j > 0; --j) {
        s = fma(-W.C(j - 1), s, W.D(j - 1));
        take(j, s);
        if (j <= iv) break;
      }
    }
  }
  const double hi = h(iv);
  const double a = y(iv);
  const double b = (y(iv + 1) - y(iv)) / hi - hi * (2.0 * ci + ci1) / 3.0;
  const double d = (ci1 - ci) / (3.0 * hi);
  const double dx = xe - x(iv);
  *val = a + b * dx + ci * (dx * dx) + d * (dx * dx * dx);
  *der = b + 2.0 * ci * dx + 3.0 * d * (dx * dx);
}

__device__ __forceinline__ void spline_at(const double* __restrict__ X, const TileView& V, int ay,
                                          int n, double xe, int iv, const SplineScratch& W,
                                          double* val, double* der) {
  spline_eval(X, [&](int i) { return V.at(ay, i); }, n, xe, iv, W, val, der);
}

// CenteredDifference first/second derivative at row i, zero outside the
// rows [1, n-2) that AmericanOptionResult::gamma fills
// (american_option_result.cpp:66-71).
__device__ __forceinline__ void stencil_at(const double* __restrict__ X, const TileView& V, int au, int n,
                           int i, bool uniform, double* d1, double* d2) {
  *d1 = 0.0;
  *d2 = 0.0;
  if (i < 1 || i >= n - 2) return;
  const double ul = V.at(au, i - 1), uc = V.at(au, i), ur = V.at(au, i + 1);
  if (uniform) {
    const double expected = (ROW(X, n - 1) - ROW(X, 0)) / static_cast<double>(n - 1);
    const double dxi = 1.0 / expected;
    const double dx2 = dxi * dxi;
    *d2 = fma(ur + ul, dx2, -2.0 * uc * dx2);
    *d1 = (ur - ul) * (dxi * 0.5);
    return;
  }
  const double dl = ROW(X, i) - ROW(X, i - 1), dr = ROW(X, i + 1) - ROW(X, i);
  const double dc = 0.5 * (dl + dr);
  const double li = 1.0 / dl, ri = 1.0 / dr, ci = 1.0 / dc;
  const double wl = dr / (dl + dr), wr = dl / (dl + dr);
  *d2 = ((ur - uc) * ri - (uc - ul) * li) * ci;
  *d1 = wl * (uc - ul) * li + wr * (ur - uc) * ri;
}


}  // namespace

// value, delta, gamma, theta of an option (american_option_result.cpp:25-121)
// from a solution on grid X: final u in array au, previous in aup, the
// option's log-moneyness xs_, strike and spot, the solve's dt.
__device__ __forceinline__ void option_outputs(const double* __restrict__ X, const TileView& V, int au, int aup,
                               int n, double xs_, double strike, double spot, double dt,
                               bool uniform, bool value_only, const SplineScratch& W,
                               double* __restrict__ res) {
  const int iv = find_interval(X, n, xs_);
  double sv, sd;
  spline_at(X, V, au, n, xs_, iv, W, &sv, &sd);
  double value;
  if (xs_ <= ROW(X, 0)) value = V.at(au, 0) * strike;
  else if (xs_ >= ROW(X, n - 1)) value = V.at(au, n - 1) * strike;
  else value = dmax_ref(0.0, sv) * strike;
  const double delta = sd * (strike / spot);
  if (value_only) {
    res[0] = value;
    res[1] = delta;
    return;
  }
  // gamma: stencil derivatives linearly interpolated at x_spot.
  int il, ir;
  if (xs_ <= ROW(X, 0)) {
    il = ir = 0;
  } else if (xs_ >= ROW(X, n - 1)) {
    il = ir = n - 1;
  } else {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = lo + (hi - lo) / 2;
      if (ROW(X, mid) < xs_) lo = mid + 1; else hi = mid;
    }
    ir = lo;
    il = ir > 0 ? ir - 1 : 0;
    if (fabs(ROW(X, ir) - xs_) < 1e-14) il = ir;
  }
  double d1l, d2l, d1r, d2r;
  stencil_at(X, V, au, n, il, uniform, &d1l, &d2l);
  double d1, d2;
  if (il == ir) {
    d1 = d1l;
    d2 = d2l;
  } else {
    stencil_at(X, V, au, n, ir, uniform, &d1r, &d2r);
    const double al = (xs_ - ROW(X, il)) / (ROW(X, ir) - ROW(X, il));
    d1 = d1l + al * (d1r - d1l);
    d2 = d2l + al * (d2r - d2l);
  }
  const double kos2 = strike / (spot * spot);
  const double gam = fma(kos2, d2, -kos2 * d1);
  // theta: (S_prev(x) - S(x)) / dt * K with an unclamped spline value.
  double pv, pd;
  spline_at(X, V, aup, n, xs_, iv, W, &pv, &pd);
  const double theta = (pv - sv) / dt * strike;
  res[0] = value;
  res[1] = delta;
  res[2] = gam;
  res[3] = theta;
}


}  // namespace mgpu
