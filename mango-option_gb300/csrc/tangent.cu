// tangent.cu -- exact discrete sensitivities of the American march by
// forward-mode (tangent-linear) differentiation.
//
// The primal is the reference's plain method on one option's own grid:
// PDESolver::solve with the Rannacher start and TR-BDF2 stages
// (src/pde/internal/pde_solver.hpp:114-178, 342-447), each stage
// solve_implicit_stage_projected (pde_solver.hpp:525-729: boundary values,
// the deep-ITM lock, solve_thomas_projected, src/math/thomas_solver.hpp:
// 321-420), the Black-Scholes operator (spatial_operator.hpp:74-163,
// black_scholes_pde.hpp:72-76) and AmericanOptionResult's value and delta
// (src/option/american_option_result.cpp:25-60, natural CubicSpline,
// src/math/cubic_spline_solver.hpp:74-230).  Beside it the kernel carries
// three tangents, d/dsigma, d/drate and d/ddividend_yield, through every
// operation of that algorithm: the operator's coefficients
// a = sigma^2/2, b = r - q - a, c = -r are linear in the stencils, the
// Thomas forward sweep is differentiated row by row (denominator, reciprocal,
// modified upper band and right-hand side), and the projected back
// substitution x_i = max(y_i, psi_i) passes the tangent of y_i where the
// obstacle is inactive and 0 where it binds (the active set and the lock rows
// of the primal, frozen).  The result is the derivative of the discrete
// price the march computes, the quantity that central differences on the
// same frozen grid approximate, in one pass; d/dstrike follows from the final
// spline alone because the log-moneyness grid does not depend on the strike.
//
// GB300 layout: three threads per option, each marching the primal with one
// tangent (sigma, rate or dividend yield): the primal is recomputed three
// times, but a thread's chain of dependent row updates is half as long and
// three times as many warps hide the memory latency of a batch of ~16k
// options.  A warp holds one direction of 32 consecutive options.  Threads
// in tiles of 32 (one per warp) with every per-thread vector interleaved
// by lane (element i of array a of lane `lane` at ((a * nmax + i) * 32 +
// lane)), so a warp's loads and stores of the same row coalesce.  The
// time-invariant row coefficients (Jacobian rows, their derivative along the
// thread's direction, stencil factors) are computed once per thread, so the
// only FP64 divide left in the time loop is the Thomas reciprocal of each
// row.  Bound by FP64 issue and HBM streaming of the per-thread state; no
// tensor cores.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "engine.hpp"

namespace mgpu {
namespace {

// One tangent per thread: three threads per option carry the primal and the
// derivative along sigma, rate and dividend yield respectively.
constexpr int kTan = 1;
constexpr int kDirs = 3;
// Interleaved per-option arrays.
enum : int {
  // TA_U: u at the step start, TA_US: the TR-BDF2 stage-1 solution
  TA_X = 0, TA_PSI, TA_U, TA_US, TA_RHS, TA_CP, TA_DP,
  TA_TU,                    // + j
  TA_TUS = TA_TU + kTan,     // + j
  TA_TRHS = TA_TUS + kTan,   // + j
  TA_TCP = TA_TRHS + kTan,   // + j
  TA_TDP = TA_TCP + kTan,    // + j
  // time-invariant row coefficients, filled once per option:
  TA_JL = TA_TDP + kTan, TA_JD, TA_JU,           // assemble_jacobian's rows
  TA_TJL, TA_TJD, TA_TJU,                        // their derivative along the direction
  TA_LI, TA_RI, TA_CI, TA_WL, TA_WR,              // CenteredDifference factors
  TA_COUNT
};

struct TanOpt {
  double S, K, T, sigma, r, q;
  int64_t x_off;
  int32_t n, nt, put, pad;
};

struct TanOut {
  double value, delta, dsigma, drate, ddiv, dstrike;
  int32_t status, pad;
};

struct View {
  double* base;
  int nmax;
  __device__ __forceinline__ double& operator()(int a, int i) const {
    return base[(static_cast<size_t>(a) * nmax + i) * 32];
  }
};

// Per-parameter derivatives of (a, b, c).
struct Coef {
  double a, b, c;
  double da[kTan], db[kTan], dc[kTan];
  double dbc;  // 1 for the rate direction (the call's right boundary moves)
};

__device__ __forceinline__ void stencil(const View& v, int arr, int i, double& d2, double& d1) {
  const double um = v(arr, i - 1), u0 = v(arr, i), up = v(arr, i + 1);
  const double li = v(TA_LI, i), ri = v(TA_RI, i);
  const double fwd = (up - u0) * ri, bwd = (u0 - um) * li;
  d2 = (fwd - bwd) * v(TA_CI, i);
  d1 = v(TA_WL, i) * (u0 - um) * li + v(TA_WR, i) * (up - u0) * ri;
}

// assemble_jacobian's row coefficients (spatial_operator.hpp:123-163) for
// operator coefficients (a, b, c).
__device__ __forceinline__ void jac_row(double dxl, double dxr, double a, double b, double c,
                                        double& jl, double& jd, double& ju) {
  const double dxa = (dxl + dxr) / 2.0;
  const double d1d = dxl + dxr;
  jl = a / (dxl * dxa) + (-b * dxr / (dxl * d1d));
  jd = (-a * (1.0 / dxl + 1.0 / dxr) / dxa) + b * (dxr - dxl) / (dxl * dxr) + c;
  ju = a / (dxr * dxa) + b * dxl / (dxr * d1d);
}

__device__ __forceinline__ double bc_right(bool put, double xr, double r, double t) {
  return put ? 0.0 : exp(xr) - exp(-r * t);
}

// One projected implicit stage with its tangents: array g holds the guess
// (read by the deep-ITM lock test only), RHS / TRHS_j the right-hand sides;
// the solution goes to array o and its tangents to to + j (o may be g: every
// read of g precedes the back substitution).
__device__ bool tan_stage(const View& v, int n, bool put, const Coef& C, double psi_max,
                          double t, double w, int g, int o, int to) {
  const double xl = v(TA_X, 0), xr = v(TA_X, n - 1);
  const double bl = put ? fmax(1.0 - exp(xl), 0.0) : 0.0;
  const double br = bc_right(put, xr, -C.c, t);
  const double dbr_dr = put ? 0.0 : t * exp(C.c * t);  // d/dr of -exp(-r t)
  const double thr = 0.95 * psi_max;
  // row 0: identity, rhs = left boundary value
  double cp = 0.0, dp = bl;
  double tcp[kTan] = {0.0}, tdp[kTan] = {0.0};
  v(TA_CP, 0) = cp;
  v(TA_DP, 0) = dp;
#pragma unroll
  for (int j = 0; j < kTan; ++j) {
    v(TA_TCP + j, 0) = 0.0;
    v(TA_TDP + j, 0) = 0.0;
  }
  // Row inputs are loaded one row ahead: none of the arrays read here is
  // written by this sweep, so the next row's loads overlap this row's work.
  struct RowIn {
    double ps, rhs, gv, jl, jd, ju, tjl, tjd, tju, trhs;
  };
  auto load_row = [&](int i) {
    RowIn r;
    r.ps = v(TA_PSI, i);
    r.rhs = v(TA_RHS, i);
    r.gv = v(g, i);
    r.jl = v(TA_JL, i);
    r.jd = v(TA_JD, i);
    r.ju = v(TA_JU, i);
    r.tjl = v(TA_TJL, i);
    r.tjd = v(TA_TJD, i);
    r.tju = v(TA_TJU, i);
    r.trhs = v(TA_TRHS, i);
    return r;
  };
  RowIn nx = load_row(1);
  for (int i = 1; i < n - 1; ++i) {
    const RowIn cu = nx;
    if (i + 1 < n - 1) nx = load_row(i + 1);
    const double ps = cu.ps;
    double lo, di, up, rhs, tlo, tdi, tup, trhs;
    bool lock = false;
    if (psi_max > 0.0 && ps > thr && cu.gv - ps < 1e-8) {
      double d2, d1;
      stencil(v, TA_PSI, i, d2, d1);
      lock = C.a * d2 + C.b * d1 + C.c * ps < 0.0;
    }
    if (lock) {
      lo = 0.0;
      di = 1.0;
      up = 0.0;
      rhs = ps;
      tlo = tdi = tup = trhs = 0.0;
    } else {
      lo = -w * cu.jl;
      di = 1.0 - w * cu.jd;
      up = -w * cu.ju;
      rhs = cu.rhs;
      tlo = -w * cu.tjl;
      tdi = -w * cu.tjd;
      tup = -w * cu.tju;
      trhs = cu.trhs;
    }
    const double denom = fma(-lo, cp, di);
    if (fabs(denom) < 1e-15) return false;
    const double inv = 1.0 / denom;
    const double num = fma(-lo, dp, rhs);
    const double ncp = up * inv, ndp = num * inv;
    const double tden = tdi - tlo * cp - lo * tcp[0];
    const double tinv = -inv * inv * tden;
    const double tnum = trhs - tlo * dp - lo * tdp[0];
    tcp[0] = tup * inv + up * tinv;
    tdp[0] = tnum * inv + num * tinv;
    v(TA_TCP, i) = tcp[0];
    v(TA_TDP, i) = tdp[0];
    cp = ncp;
    dp = ndp;
    v(TA_CP, i) = cp;
    v(TA_DP, i) = dp;
  }
  // row n-1: identity, rhs = right boundary value
  const double dpl = br;
  const double tdpl[kTan] = {C.dbc * dbr_dr};
  // projected back substitution
  double x = fmax(dpl, v(TA_PSI, n - 1));
  double tx[kTan];
  const bool act_l = dpl < v(TA_PSI, n - 1);
#pragma unroll
  for (int j = 0; j < kTan; ++j) tx[j] = act_l ? 0.0 : tdpl[j];
  double nc = v(TA_CP, n - 2), nd = v(TA_DP, n - 2), nps = v(TA_PSI, n - 2);
  double ntd = v(TA_TDP, n - 2), ntc = v(TA_TCP, n - 2);
  for (int i = n - 2; i >= 0; --i) {
    const double c = nc, d = nd, ps = nps, td = ntd, tc = ntc;
    if (i > 0) {  // next row's inputs (this sweep writes only o and to)
      nc = v(TA_CP, i - 1);
      nd = v(TA_DP, i - 1);
      nps = v(TA_PSI, i - 1);
      ntd = v(TA_TDP, i - 1);
      ntc = v(TA_TCP, i - 1);
    }
    const double unc = fma(-c, x, d);
    const bool act = unc < ps;
    tx[0] = act ? 0.0 : td - tc * x - c * tx[0];
    v(to, i) = tx[0];
    x = act ? ps : unc;
    v(o, i) = x;
  }
  // boundary values again
  v(o, 0) = bl;
  v(o, n - 1) = br;
#pragma unroll
  for (int j = 0; j < kTan; ++j) {
    v(to + j, 0) = 0.0;
    v(to + j, n - 1) = tdpl[j];
  }
  return true;
}

// Natural cubic spline of array y on X at xs (CubicSpline::build / eval /
// eval_derivative); uses TA_RHS, TA_CP, TA_DP as scratch.
__device__ bool spline_at(const View& v, int n, int y, double xs, double& val, double& der) {
  const int m = n - 2;
  auto h = [&](int k) { return v(TA_X, k + 1) - v(TA_X, k); };
  // tridiagonal system for the interior second-derivative coefficients
  double cp = 0.0, dp = 0.0;
  for (int i = 0; i < m; ++i) {
    const int k = i + 1;
    const double td = 2.0 * (h(k - 1) + h(k));
    const double tl = h(k - 1), tu = h(k);
    const double sr = (v(y, k + 1) - v(y, k)) / h(k);
    const double sl = (v(y, k) - v(y, k - 1)) / h(k - 1);
    const double tr = 3.0 * (sr - sl);
    if (i == 0) {
      if (fabs(td) < 1e-15) return false;
      cp = tu / td;
      dp = tr / td;
    } else if (i < m - 1) {
      const double denom = fma(-tl, cp, td);
      if (fabs(denom) < 1e-15) return false;
      const double inv = 1.0 / denom;
      dp = fma(-tl, dp, tr) * inv;
      cp = tu * inv;
    } else {
      const double denom = fma(-tl, cp, td);
      if (fabs(denom) < 1e-15) return false;
      dp = fma(-tl, dp, tr) / denom;
    }
    v(TA_CP, i) = cp;
    v(TA_DP, i) = dp;
  }
  // c[0] = c[n-1] = 0, c[i+1] = solution i
  v(TA_RHS, 0) = 0.0;
  v(TA_RHS, n - 1) = 0.0;
  double s = v(TA_DP, m - 1);
  v(TA_RHS, m) = s;
  for (int i = m - 1; i > 0; --i) {
    s = fma(-v(TA_CP, i - 1), s, v(TA_DP, i - 1));
    v(TA_RHS, i) = s;
  }
  // find_interval (lower_bound semantics)
  int idx;
  if (xs <= v(TA_X, 0)) {
    idx = 0;
  } else if (xs >= v(TA_X, n - 1)) {
    idx = n - 2;
  } else {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = lo + (hi - lo) / 2;
      if (v(TA_X, mid) < xs) lo = mid + 1; else hi = mid;
    }
    idx = lo;
    if (idx > 0 && (idx == n || v(TA_X, idx) > xs)) --idx;
    idx = min(idx, n - 2);
  }
  const double hi_ = h(idx);
  const double c0 = v(TA_RHS, idx), c1 = v(TA_RHS, idx + 1);
  const double a = v(y, idx);
  const double b = (v(y, idx + 1) - a) / hi_ - hi_ * (2.0 * c0 + c1) / 3.0;
  const double d = (c1 - c0) / (3.0 * hi_);
  const double dx = xs - v(TA_X, idx);
  val = a + b * dx + c0 * (dx * dx) + d * (dx * dx * dx);
  der = b + 2.0 * c0 * dx + 3.0 * d * (dx * dx);
  return true;
}

__global__ void __launch_bounds__(128) tangent_march_kernel(const TanOpt* __restrict__ opts, int n_opts,
                                                            const double* __restrict__ xs_all,
                                                            double* __restrict__ ws, int nmax,
                                                            TanOut* __restrict__ out) {
  // warp w holds direction w % kDirs of options (w / kDirs) * 32 + lane
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int w = k / 32, lane = k % 32;
  const int dir = w % kDirs;
  const int oi = (w / kDirs) * 32 + lane;
  if (oi >= n_opts) return;
  const int ko = oi * kDirs + dir;  // result slot
  const TanOpt o = opts[oi];
  TanOut res{};
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  res.value = res.delta = res.dsigma = res.drate = res.ddiv = res.dstrike = nan;
  if (o.n < 3 || o.n > nmax || o.nt < 1) {
    res.status = MANGO_ERR_VALIDATION;
    out[ko] = res;
    return;
  }
  View v{ws + static_cast<size_t>(w) * TA_COUNT * nmax * 32 + lane, nmax};
  const int n = o.n;
  const bool put = o.put != 0;
  Coef C;
  C.a = 0.5 * o.sigma * o.sigma;
  C.b = o.r - o.q - C.a;
  C.c = -o.r;
  // direction 0: sigma (da = sigma, db = -sigma), 1: rate (db = 1, dc = -1),
  // 2: dividend yield (db = -1)
  C.da[0] = dir == 0 ? o.sigma : 0.0;
  C.db[0] = dir == 0 ? -o.sigma : (dir == 1 ? 1.0 : -1.0);
  C.dc[0] = dir == 1 ? -1.0 : 0.0;
  C.dbc = dir == 1 ? 1.0 : 0.0;
  double psi_max = 0.0;
  for (int i = 0; i < n; ++i) {
    const double x = xs_all[o.x_off + i];
    v(TA_X, i) = x;
    const double ps = put ? fmax(1.0 - exp(x), 0.0) : fmax(exp(x) - 1.0, 0.0);
    v(TA_PSI, i) = ps;
    psi_max = i == 0 ? ps : fmax(psi_max, ps);
  }
  for (int i = 1; i < n - 1; ++i) {
    const double dxl = v(TA_X, i) - v(TA_X, i - 1);
    const double dxr = v(TA_X, i + 1) - v(TA_X, i);
    double jl, jd, ju;
    jac_row(dxl, dxr, C.a, C.b, C.c, jl, jd, ju);
    v(TA_JL, i) = jl;
    v(TA_JD, i) = jd;
    v(TA_JU, i) = ju;
    // the rows are linear in (a, b, c): the same formula on (da, db, dc)
    jac_row(dxl, dxr, C.da[0], C.db[0], C.dc[0], jl, jd, ju);
    v(TA_TJL, i) = jl;
    v(TA_TJD, i) = jd;
    v(TA_TJU, i) = ju;
    v(TA_LI, i) = 1.0 / dxl;
    v(TA_RI, i) = 1.0 / dxr;
    v(TA_CI, i) = 1.0 / (0.5 * (dxl + dxr));
    v(TA_WL, i) = dxr / (dxl + dxr);
    v(TA_WR, i) = dxl / (dxl + dxr);
  }
  // initialize: payoff, boundary values at t = 0, obstacle
  const double bl0 = put ? fmax(1.0 - exp(v(TA_X, 0)), 0.0) : 0.0;
  const double br0 = bc_right(put, v(TA_X, n - 1), o.r, 0.0);
  for (int i = 0; i < n; ++i) {
    double u = v(TA_PSI, i);
    if (i == 0) u = bl0;
    if (i == n - 1) u = br0;
    v(TA_U, i) = fmax(u, v(TA_PSI, i));
#pragma unroll
    for (int j = 0; j < kTan; ++j) v(TA_TU + j, i) = 0.0;
  }
  const double dt = o.T / static_cast<double>(o.nt);
  const double gamma = 2.0 - sqrt(2.0);
  bool ok = true;
  // Rannacher start: two implicit-Euler half steps
  {
    const double half = 0.5 * dt;
    for (int hs = 0; hs < 2 && ok; ++hs) {
      for (int i = 0; i < n; ++i) {
        v(TA_RHS, i) = v(TA_U, i);
#pragma unroll
        for (int j = 0; j < kTan; ++j) v(TA_TRHS + j, i) = v(TA_TU + j, i);
      }
      ok = tan_stage(v, n, put, C, psi_max, hs == 0 ? half : dt, half, TA_U, TA_U, TA_TU);
    }
  }
  double t = dt;
  const double w1 = gamma * dt / 2.0;
  const double omg = 1.0 - gamma, tmg = 2.0 - gamma, den = gamma * tmg;
  const double alpha = 1.0 / den, beta = -(omg * omg) / den;
  const double w2 = (1.0 - gamma) * dt / (2.0 - gamma);
  for (int step = 1; ok && step < o.nt; ++step) {
    const double t_next = static_cast<double>(step + 1) * dt;
    // stage 1: rhs = u + w1 L(u), guess u, solution into US (u stays in U)
    for (int i = 0; i < n; ++i) {
      const double u = v(TA_U, i);
      double lu = 0.0, tl[kTan] = {0.0};
      if (i > 0 && i < n - 1) {
        const double li = v(TA_LI, i), ri = v(TA_RI, i), ci = v(TA_CI, i);
        const double wl = v(TA_WL, i), wr = v(TA_WR, i);
        const double um = v(TA_U, i - 1), upl = v(TA_U, i + 1);
        const double d2 = ((upl - u) * ri - (u - um) * li) * ci;
        const double d1 = wl * (u - um) * li + wr * (upl - u) * ri;
        lu = C.a * d2 + C.b * d1 + C.c * u;
#pragma unroll
        for (int j = 0; j < kTan; ++j) {
          const double tm = v(TA_TU + j, i - 1), t0 = v(TA_TU + j, i), tp = v(TA_TU + j, i + 1);
          const double e2 = ((tp - t0) * ri - (t0 - tm) * li) * ci;
          const double e1 = wl * (t0 - tm) * li + wr * (tp - t0) * ri;
          tl[j] = C.da[j] * d2 + C.db[j] * d1 + C.dc[j] * u + C.a * e2 + C.b * e1 + C.c * t0;
        }
      }
      v(TA_RHS, i) = fma(w1, lu, u);
#pragma unroll
      for (int j = 0; j < kTan; ++j) v(TA_TRHS + j, i) = w1 * tl[j] + v(TA_TU + j, i);
    }
    ok = tan_stage(v, n, put, C, psi_max, t + gamma * dt, w1, TA_U, TA_US, TA_TUS);
    if (!ok) break;
    // stage 2: rhs = alpha u* + beta u, guess u*, solution into U
    for (int i = 0; i < n; ++i) {
      v(TA_RHS, i) = fma(alpha, v(TA_US, i), beta * v(TA_U, i));
#pragma unroll
      for (int j = 0; j < kTan; ++j)
        v(TA_TRHS + j, i) = alpha * v(TA_TUS + j, i) + beta * v(TA_TU + j, i);
    }
    ok = tan_stage(v, n, put, C, psi_max, t_next, w2, TA_US, TA_U, TA_TU);
    t = t_next;
  }
  if (!ok) {
    res.status = MANGO_ERR_SOLVER;
    out[ko] = res;
    return;
  }
  // AmericanOptionResult::value_at / delta and the tangents' splines
  const double xs = log(o.S / o.K);
  double s, sd;
  if (!spline_at(v, n, TA_U, xs, s, sd)) {
    res.status = MANGO_ERR_SOLVER;
    out[ko] = res;
    return;
  }
  double tv, tdj;
  if (!spline_at(v, n, TA_TU, xs, tv, tdj)) {
    res.status = MANGO_ERR_SOLVER;
    out[ko] = res;
    return;
  }
  double value, dK;
  if (xs <= v(TA_X, 0) || xs >= v(TA_X, n - 1)) {
    const int e = xs <= v(TA_X, 0) ? 0 : n - 1;
    value = v(TA_U, e) * o.K;
    tv = v(TA_TU, e);
    dK = v(TA_U, e);
  } else {
    const bool pos = 0.0 < s;
    value = (pos ? s : 0.0) * o.K;
    tv = pos ? tv : 0.0;
    dK = pos ? s - sd : 0.0;
  }
  // each thread reports the primal and its own direction in dsigma
  res.value = value;
  res.delta = sd * (o.K / o.S);
  res.dsigma = tv * o.K;
  res.dstrike = dK;
  res.status = MANGO_OK;
  out[ko] = res;
}

}  // namespace
}  // namespace mgpu

using namespace mgpu;

extern "C" MangoStatus mango_gpu_price_american_tangent_batch(
    MangoGpuContext* ctx, const MangoPricingParams* params, uint64_t n, const MangoGpuGrid* grids,
    uint64_t grid_stride, MangoGpuGreeksOut* out, uint64_t* out_failed, MangoError* err) {
  if (!ctx || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, params or out");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 26)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^26 options");
    return MANGO_ERR_VALIDATION;
  }
  if (out_failed) *out_failed = 0;
  if (n == 0) return MANGO_OK;
  DevBuf d_opts, d_x, d_ws, d_out;
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const int64_t nn = static_cast<int64_t>(n);
    std::vector<Resolved> res(static_cast<size_t>(nn));
    std::vector<std::string> msg(static_cast<size_t>(nn));
    parallel_for(nn, [&](int64_t i) {
      thread_local std::vector<double> scratch;
      std::string m = validate(params[i], false);
      if (m.empty()) {
        MangoGpuGrid g{};
        g.kind = MANGO_GPU_GRID_AUTO;
        if (grids) g = grids[grid_stride ? i : 0];
        m = resolve(params[i], g, &res[i], &scratch);
      }
      if (!m.empty()) {
        res[i].status = MANGO_ERR_VALIDATION;
        msg[i] = m;
      }
    });
    std::vector<TanOpt> opts(static_cast<size_t>(nn));
    std::vector<int64_t> xoff(static_cast<size_t>(nn) + 1, 0);
    int nmax = 3;
    for (int64_t i = 0; i < nn; ++i) {
      const int64_t np = res[i].status == 0 ? res[i].spec.n : 0;
      xoff[i + 1] = xoff[i] + np;
      nmax = std::max<int>(nmax, static_cast<int>(np));
    }
    std::vector<double> xs(static_cast<size_t>(std::max<int64_t>(xoff[nn], 1)));
    parallel_for(nn, [&](int64_t i) {
      const MangoPricingParams& p = params[i];
      TanOpt& o = opts[i];
      o.S = p.spot; o.K = p.strike; o.T = p.maturity; o.sigma = p.volatility;
      o.r = p.rate_const; o.q = p.dividend_yield;
      o.put = p.option_type == MANGO_PUT ? 1 : 0;
      o.x_off = xoff[i];
      if (res[i].status == 0) {
        generate_grid(res[i].spec, xs.data() + xoff[i]);
        o.n = static_cast<int32_t>(res[i].spec.n);
        o.nt = static_cast<int32_t>(res[i].nt);
      } else {
        o.n = 0;  // rejected on the device as invalid, overwritten below
        o.nt = 0;
      }
    }, 64);
    d_opts.get(sizeof(TanOpt) * n);
    d_x.get(sizeof(double) * xs.size());
    d_out.get(sizeof(TanOut) * n * kDirs);
    check(cudaMemcpyAsync(d_opts.p, opts.data(), sizeof(TanOpt) * n, cudaMemcpyHostToDevice, st), "H2D");
    check(cudaMemcpyAsync(d_x.p, xs.data(), sizeof(double) * xs.size(), cudaMemcpyHostToDevice, st), "H2D");
    // workspace chunks of at most 4 GiB
    const size_t per_tile = static_cast<size_t>(TA_COUNT) * nmax * 32 * sizeof(double);
    const int64_t tiles_per_chunk = std::max<int64_t>(1, static_cast<int64_t>((size_t{4} << 30) / per_tile));
    const int64_t ntiles = (nn + 31) / 32 * kDirs;
    const int64_t chunk_tiles = std::min(ntiles, std::max<int64_t>(tiles_per_chunk, kDirs));
    d_ws.get(per_tile * static_cast<size_t>(chunk_tiles));
    // options per chunk: their kDirs threads fill at most chunk_tiles tiles
    const int64_t per_chunk = std::max<int64_t>(1, chunk_tiles / kDirs) * 32;
    for (int64_t o0 = 0; o0 < nn; o0 += per_chunk) {
      const int cnt = static_cast<int>(std::min<int64_t>(nn - o0, per_chunk));
      const int threads = (cnt + 31) / 32 * 32 * kDirs;
      tangent_march_kernel<<<(threads + 127) / 128, 128, 0, st>>>(
          d_opts.as<TanOpt>() + o0, cnt, d_x.as<double>(), d_ws.as<double>(), nmax,
          d_out.as<TanOut>() + o0 * kDirs);
      check(cudaGetLastError(), "tangent_march_kernel launch");
    }
    std::vector<TanOut> ho(static_cast<size_t>(nn) * kDirs);
    check(cudaMemcpyAsync(ho.data(), d_out.p, sizeof(TanOut) * n * kDirs, cudaMemcpyDeviceToHost, st),
          "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    uint64_t failed = 0;
    std::string first;
    const double nan = std::nan("");
    for (int64_t i = 0; i < nn; ++i) {
      MangoGpuGreeksOut& g = out[i];
      MangoGpuAmericanOut& b = g.base;
      const TanOut& h = ho[kDirs * i];
      const TanOut& hr = ho[kDirs * i + 1];
      const TanOut& hq = ho[kDirs * i + 2];
      g = MangoGpuGreeksOut{};
      b.status = res[i].status != 0 ? res[i].status
                                    : (h.status != 0 ? h.status : (hr.status != 0 ? hr.status : hq.status));
      b.n_space = static_cast<int32_t>(res[i].spec.n);
      b.n_time = static_cast<int32_t>(res[i].nt);
      b.gamma = b.theta = nan;
      if (b.status != MANGO_OK) {
        b.value = b.delta = g.vega = g.rho = g.dividend_rho = g.dstrike = nan;
        if (failed++ == 0) first = msg[i].empty() ? "solver failure" : msg[i];
        continue;
      }
      b.value = h.value;
      b.delta = h.delta;
      g.vega = h.dsigma;
      g.rho = hr.dsigma;
      g.dividend_rho = hq.dsigma;
      g.dstrike = h.dstrike;
    }
    if (out_failed) *out_failed = failed;
    d_opts.release(); d_x.release(); d_ws.release(); d_out.release();
    if (failed == n) {
      set_err(err, MANGO_ERR_VALIDATION, "every option failed: " + first);
      return MANGO_ERR_VALIDATION;
    }
    return MANGO_OK;
  } catch (const std::exception& e) {
    d_opts.release(); d_x.release(); d_ws.release(); d_out.release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}
