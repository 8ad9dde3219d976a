// march_tv.cu -- the American-option march for options whose stage matrices
// change during the solve: a yield curve (a piecewise-constant forward rate
// r(t)), discrete dividends (mandatory time points, so the step changes, and
// a spline shift of the solution at every ex-dividend time), or both.
//
// Restates, per option, PDESolver::solve (src/pde/internal/pde_solver.hpp:
// 114-178) with time-dependent coefficients:
//   * stage 1 takes L(u^n) at t_n and the stage matrix at t_n + gamma dt,
//     stage 2 its matrix at t_{n+1}, the Rannacher half steps theirs at
//     t + dt/2 and t + dt (pde_solver.hpp:342-447), each through
//     solve_implicit_stage_projected (pde_solver.hpp:525-729) with the
//     analytic Jacobian at that time (spatial_operator.hpp:123-163) and the
//     deep-ITM lock tested with L(psi) at that time;
//   * r(t) = YieldCurve::rate(max(0, T - t)) and the call's right boundary
//     e^x - D(T)/D(T - t) (src/option/option_spec.hpp:50-91,
//     src/option/yield_curve.hpp:105-130);
//   * temporal events after each step in (t_old, t_new]
//     (pde_solver.hpp:244-275): the dividend shift u(x) <- u(ln(e^x - D/K))
//     through a natural cubic spline of u (american_option.cpp:83-144),
//     then the boundary values and the obstacle.
//
// GB300 design.  The cached-factorisation march (march.cu) needs one matrix
// per stage for the whole solve; here every stage refactors its matrix, so
// each row costs two reciprocals more.  The grid-only parts of every
// coefficient (second-derivative weights, first-derivative multipliers,
// centred-difference weights, derivatives of psi) are computed once per
// option into the tile block, so a stage forms its bands with a few FMAs.
// One lane per option, one warp per tile of 32, lanes of a tile share n and
// move through the rows together, so every row access is one coalesced
// 256-byte warp load.
#include <cuda_runtime.h>

#include <cstdint>

#include "march.cuh"

namespace mgpu {

namespace {

// Roles of the tile arrays on this march (the cached march's stencil and
// factor slots are free here).
enum : int {
  T_D2M = A_E1L,  // a/(dxl dxa): second-derivative weight of u_{i-1}
  T_D2I = A_E1D,  // -a(1/dxl + 1/dxr)/dxa
  T_D2P = A_E1U,  // a/(dxr dxa)
  T_QM = A_N1H,   // dxr/(dxl (dxl + dxr)): d1 weight of u_{i-1} per unit of b
  T_QI = A_NC1,   // (dxr - dxl)/(dxl dxr)
  T_QP = A_A2H,   // dxl/(dxr (dxl + dxr))
  T_LI = A_B2H,   // 1/dxl      (CenteredDifference on a non-uniform grid)
  T_RI = A_N2H,   // 1/dxr
  T_CI = A_NC2,   // 1/((dxl + dxr)/2)
  T_WL = A_E1L0,  // dxr/(dxl + dxr)
  T_WR = A_E1D0,  // dxl/(dxl + dxr)
  T_D2PSI = A_E1U0,  // second derivative of psi (time invariant)
  T_D1PSI = A_L1,    // first derivative of psi
  T_SPC = A_D1,      // dividend spline: second-derivative terms c_i
  T_SPY = A_D2,      // dividend spline: the knot values
};

// YieldCurve over (tenor, log discount) pairs sorted by tenor.
struct Curve {
  const double* p;
  int n;
  __device__ __forceinline__ double tenor(int j) const { return p[2 * j]; }
  __device__ __forceinline__ double ld(int j) const { return p[2 * j + 1]; }
  // std::upper_bound on the tenors: the first j with t < tenor_j.
  __device__ int upper(double t) const {
    int lo = 0, hi = n;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (t < tenor(mid)) hi = mid; else lo = mid + 1;
    }
    return lo;
  }
  // YieldCurve::rate_between
  __device__ double rate_between(int idx) const {
    if (idx + 1 >= n) return 0.0;
    const double dt = __dsub_rn(tenor(idx + 1), tenor(idx));
    if (dt <= 0.0) return 0.0;
    return -(__dsub_rn(ld(idx + 1), ld(idx)) / dt);
  }
  // YieldCurve::rate: the forward rate of the tenor interval holding t.
  __device__ double rate(double t) const {
    if (n < 2) return 0.0;
    if (t <= 0.0) return rate_between(0);
    const int j = upper(t);
    if (j == 0) return rate_between(0);
    if (j == n) return rate_between(n - 2);
    return rate_between(j - 1);
  }
  // YieldCurve::log_discount: linear in t between tenors, flat forward rate
  // beyond the last one.
  __device__ double log_discount(double t) const {
    if (n < 2) return 0.0;
    if (t <= 0.0) return 0.0;
    const int j = upper(t);
    if (j == 0) return 0.0;
    if (j == n) {
      const double rate = -(__dsub_rn(ld(n - 1), ld(n - 2)) / __dsub_rn(tenor(n - 1), tenor(n - 2)));
      return __dsub_rn(ld(n - 1), __dmul_rn(rate, __dsub_rn(t, tenor(n - 1))));
    }
    const double alpha = __dsub_rn(t, tenor(j - 1)) / __dsub_rn(tenor(j), tenor(j - 1));
    return __dadd_rn(ld(j - 1), __dmul_rn(alpha, __dsub_rn(ld(j), ld(j - 1))));
  }
};

struct Lane {
  TileView V;
  const double* X;
  int n;
  bool put;
  bool uniform;
  double hss, q;
  double u_dx2, u_hdx;  // uniform-grid centred-difference weights
  double psi_max, thr;
  int clo, chi;         // interior rows with psi > thr (lock candidates): [clo, chi]
  double bcl;           // left boundary value (time invariant)
  double exp_xr;        // e^{x_{n-1}}
  double T, r_const;
  Curve curve;

  __device__ __forceinline__ double x(int i) const { return ROW(X, i); }
  // make_rate_fn: r at time-to-expiry tau.
  __device__ double rate(double tau) const {
    if (curve.n == 0) return r_const;
    return curve.rate(dmax_ref(0.0, __dsub_rn(T, tau)));
  }
  // Right boundary value: put 0, call e^x - forward discount to expiry.
  __device__ double bcr(double tau) const {
    if (put) return 0.0;
    double disc;
    if (curve.n == 0) {
      disc = exp(-r_const * tau);
    } else {
      const double s = dmax_ref(0.0, __dsub_rn(T, tau));
      disc = exp(curve.log_discount(T)) / exp(curve.log_discount(s));
    }
    return __dsub_rn(exp_xr, disc);
  }
};

// Centred first and second differences of array a at interior row i
// (CenteredDifference, centered_difference.hpp:24-99), from the row values
// ul, uc, ur.
__device__ __forceinline__ void cdiff(const Lane& L, int i, double ul, double uc, double ur,
                                      double* d1, double* d2) {
  if (L.uniform) {
    *d2 = fma(ur + ul, L.u_dx2, -2.0 * uc * L.u_dx2);
    *d1 = (ur - ul) * L.u_hdx;
  } else {
    const double* r = L.V.rp(i);
    const double li = r[T_LI * kTile], ri = r[T_RI * kTile];
    const double fwd = (ur - uc) * ri;
    const double bwd = (uc - ul) * li;
    *d2 = (fwd - bwd) * r[T_CI * kTile];
    *d1 = r[T_WL * kTile] * (uc - ul) * li + r[T_WR * kTile] * (ur - uc) * ri;
  }
}

// Grid-only coefficients, psi, u^0 (PDESolver::initialize: payoff, boundary
// values at t = 0, obstacle) and u_prev = u^0.
__device__ void tv_setup(Lane& L) {
  const int n = L.n;
  const TileView& V = L.V;
  const double expected = (L.x(n - 1) - L.x(0)) / static_cast<double>(n - 1);
  bool uniform = true;
  for (int i = 1; i < n; ++i)
    if (fabs((L.x(i) - L.x(i - 1)) - expected) > 100.0 * 2.220446049250313e-16) {
      uniform = false;
      break;
    }
  L.uniform = uniform;
  const double u_dx_inv = 1.0 / expected;
  L.u_dx2 = u_dx_inv * u_dx_inv;
  L.u_hdx = u_dx_inv * 0.5;
  double psi_max = 0.0;
  for (int i = 0; i < n; ++i) {
    const double ex = exp(L.x(i));
    const double p = L.put ? dmax_ref(1.0 - ex, 0.0) : dmax_ref(ex - 1.0, 0.0);
    V.at(A_PSI, i) = p;
    if (i == 0 || psi_max < p) psi_max = p;
  }
  L.psi_max = psi_max;
  L.thr = 0.95 * psi_max;
  // Lock condition 1 (psi > 0.95 max psi) does not change in time: the
  // stages test the other two only on rows where it holds.
  L.clo = 0x7fffffff;
  L.chi = -1;
  if (psi_max > 0.0)
    for (int i = 1; i < n - 1; ++i)
      if (V.at(A_PSI, i) > L.thr) {
        L.clo = min(L.clo, i);
        L.chi = i;
      }
  const double a = L.hss;
  for (int i = 1; i < n - 1; ++i) {
    const double xl = L.x(i - 1), xi = L.x(i), xr = L.x(i + 1);
    const double dxl = xi - xl, dxr = xr - xi;
    const double dxa = (dxl + dxr) / 2.0;
    const double d1d = dxl + dxr;
    double* r = V.rp(i);
    r[T_D2M * kTile] = a / (dxl * dxa);
    r[T_D2I * kTile] = -a * (1.0 / dxl + 1.0 / dxr) / dxa;
    r[T_D2P * kTile] = a / (dxr * dxa);
    r[T_QM * kTile] = dxr / (dxl * d1d);
    r[T_QI * kTile] = (dxr - dxl) / (dxl * dxr);
    r[T_QP * kTile] = dxl / (dxr * d1d);
    const double dc = 0.5 * (dxl + dxr);
    r[T_LI * kTile] = 1.0 / dxl;
    r[T_RI * kTile] = 1.0 / dxr;
    r[T_CI * kTile] = 1.0 / dc;
    r[T_WL * kTile] = dxr / (dxl + dxr);
    r[T_WR * kTile] = dxl / (dxl + dxr);
  }
  for (int i = 1; i < n - 1; ++i) {
    double d1, d2;
    cdiff(L, i, V.at(A_PSI, i - 1), V.at(A_PSI, i), V.at(A_PSI, i + 1), &d1, &d2);
    V.at(T_D2PSI, i) = d2;
    V.at(T_D1PSI, i) = d1;
  }
  for (int i = 1; i < n - 1; ++i) V.at(A_G, i) = V.at(A_PSI, i);
  V.at(A_G, 0) = dmax_ref(L.bcl, V.at(A_PSI, 0));
  V.at(A_G, n - 1) = dmax_ref(L.bcr(0.0), V.at(A_PSI, n - 1));
  for (int i = 0; i < n; ++i) V.at(A_U, i) = V.at(A_G, i);
}

enum StageKind { kEuler = 0, kTrap = 1, kBdf2 = 2 };

// std::max(v, psi) for a payoff psi >= +0, by integer compare (no FP64
// instruction): non-negative doubles order like their bit patterns and a
// negative v loses.  Differs from the reference only for v = -0, psi = +0
// (+0 instead of -0, the same number).
__device__ __forceinline__ double pmax(double v, double psi) {
  const long long vb = __double_as_longlong(v), pb = __double_as_longlong(psi);
  return __longlong_as_double(vb > pb ? vb : pb);
}

// Inputs of forward-sweep row i: the grid-only band parts, psi and the
// stage's state (u_prev at row i + 1 for kEuler / kTrap, u* and u_prev at
// row i for kBdf2).
struct FwdRow {
  double d2m, d2i, d2p, qm, qi, qp, psi, s0, s1;
};
template <int KIND>
__device__ __forceinline__ FwdRow fwd_load(const TileView& V, int i) {
  const double* r = V.rp(i);
  FwdRow o;
  o.d2m = r[T_D2M * kTile];
  o.d2i = r[T_D2I * kTile];
  o.d2p = r[T_D2P * kTile];
  o.qm = r[T_QM * kTile];
  o.qi = r[T_QI * kTile];
  o.qp = r[T_QP * kTile];
  o.psi = r[A_PSI * kTile];
  if (KIND != kBdf2) {
    o.s0 = V.rp(i + 1)[A_G * kTile];
    o.s1 = 0.0;
  } else {
    o.s0 = r[A_G * kTile];
    o.s1 = r[A_U * kTile];
  }
  return o;
}
struct BwdRow {
  double cp, d, psi;
};
__device__ __forceinline__ BwdRow bwd_load(const TileView& V, int i) {
  const double* r = V.rp(i);
  return BwdRow{r[A_CP * kTile], r[A_D * kTile], r[A_PSI * kTile]};
}

// One implicit stage (solve_implicit_stage_projected) at time t_impl with
// weight w, ending in A_G.
//   kEuler: rhs = guess = u_prev, u_prev <- u first (A_G copied to A_U);
//   kTrap:  rhs = u_prev + w L(u_prev) with L at rate r_expl, guess = u_prev,
//           u_prev <- u first;
//   kBdf2:  rhs = alpha u* + beta u_prev (u* in A_G), guess = u*.
// L(u_prev) is applied in band form, the Jacobian entries at r_expl (the
// same operator as the reference's centred differences, summed in another
// order).  Both sweeps read their rows two ahead of the row being solved, so
// the serial recurrences overlap the loads.  Returns false on a pivot below
// the reference's singularity tolerance.
template <int KIND>
__device__ bool tv_stage(const Lane& L, double t_impl, double w, double r_expl, double alpha,
                         double beta) {
  const int n = L.n;
  const TileView& V = L.V;
  const double r_impl = L.rate(t_impl);
  const double b = r_impl - L.q - L.hss;  // first_derivative_coeff(t)
  const double c = -r_impl;               // -discount_rate(t)
  const double be = r_expl - L.q - L.hss;
  const double ce = -r_expl;
  const double bcl = L.bcl, bcr = L.bcr(t_impl);
  // row 0: Dirichlet identity row, rhs = boundary value
  double cp = 0.0 / 1.0;
  double dp = bcl / 1.0;
  double ul = 0.0, uc = 0.0;
  if (KIND != kBdf2) {
    ul = V.at(A_G, 0);
    uc = V.at(A_G, 1);
    V.at(A_U, 0) = ul;
    V.at(A_U, 1) = uc;
  }
  const int last = n - 2;  // last interior row
  FwdRow f0 = fwd_load<KIND>(V, 1);
  FwdRow f1 = last >= 2 ? fwd_load<KIND>(V, 2) : f0;
  for (int i = 1; i <= last; ++i) {
    const FwdRow f2 = i + 2 <= last ? fwd_load<KIND>(V, i + 2) : f1;
    double rhs, guess;
    if (KIND != kBdf2) {
      const double ur = f0.s0;
      V.at(A_U, i + 1) = ur;
      guess = uc;
      if (KIND == kTrap) {
        const double el = f0.d2m + (-be) * f0.qm;
        const double ed = f0.d2i + be * f0.qi + ce;
        const double eu = f0.d2p + be * f0.qp;
        const double lu = fma(el, ul, fma(ed, uc, eu * ur));
        rhs = fma(w, lu, uc);
      } else {
        rhs = uc;
      }
      ul = uc;
      uc = ur;
    } else {
      guess = f0.s0;
      rhs = fma(alpha, f0.s0, beta * f0.s1);
    }
    const double jl = f0.d2m + (-b) * f0.qm;
    const double jd = f0.d2i + b * f0.qi + c;
    const double ju = f0.d2p + b * f0.qp;
    double lo = -w * jl, dg = 1.0 - w * jd, up = -w * ju;
    const double psi = f0.psi;
    if (i >= L.clo && i <= L.chi && psi > L.thr && guess - psi < 1e-8) {
      const double lpsi = L.hss * V.at(T_D2PSI, i) + b * V.at(T_D1PSI, i) - r_impl * psi;
      if (lpsi < 0.0) {
        lo = 0.0;
        dg = 1.0;
        up = 0.0;
        rhs = psi;
      }
    }
    const double denom = fma(-lo, cp, dg);
    if (fabs(denom) < 1e-15) return false;
    const double inv = 1.0 / denom;
    cp = up * inv;
    dp = fma(-lo, dp, rhs) * inv;
    V.at(A_CP, i) = cp;
    V.at(A_D, i) = dp;
    f0 = f1;
    f1 = f2;
  }
  // row n-1: Dirichlet identity row (lower entry 0)
  const double dlast = fma(-0.0, dp, bcr) / fma(-0.0, cp, 1.0);
  double sol = pmax(dlast, V.at(A_PSI, n - 1));
  V.at(A_G, n - 1) = sol;
  BwdRow g0 = bwd_load(V, last);
  BwdRow g1 = last >= 2 ? bwd_load(V, last - 1) : g0;
  for (int i = last; i >= 1; --i) {
    const BwdRow g2 = i - 2 >= 1 ? bwd_load(V, i - 2) : g1;
    sol = pmax(fma(-g0.cp, sol, g0.d), g0.psi);
    V.at(A_G, i) = sol;
    g0 = g1;
    g1 = g2;
  }
  // row 0 (c'_0 = 0, d'_0 = bcl), then the boundary values again
  V.at(A_G, 0) = bcl;
  V.at(A_G, n - 1) = bcr;
  return true;
}

// Dividend shift of A_G by d = D/K (make_dividend_event): a natural cubic
// spline through the current solution (CubicSpline::rebuild_same_grid,
// cubic_spline_solver.hpp:153-179, 264-346) evaluated at ln(e^x - d), the
// intrinsic fallback below the grid; then the boundary values at the event
// time and the obstacle (pde_solver.hpp:244-275).
__device__ void tv_dividend(const Lane& L, double tau, double d, double fallback) {
  const int n = L.n;
  const TileView& V = L.V;
  auto h = [&](int i) { return L.x(i + 1) - L.x(i); };
  bool ok = true;
  if (d > 0.0) {
    for (int i = 0; i < n; ++i) V.at(T_SPY, i) = V.at(A_G, i);
    auto y = [&](int i) { return V.at(T_SPY, i); };
    V.at(T_SPC, 0) = 0.0;
    V.at(T_SPC, n - 1) = 0.0;
    const int m = n - 2;
    auto rhs = [&](int j) {  // row j, knot k = j + 1
      const int k = j + 1;
      const double sr = (y(k + 1) - y(k)) / h(k);
      const double sl = (y(k) - y(k - 1)) / h(k - 1);
      return 3.0 * (sr - sl);
    };
    if (m == 1) {
      const double dg = 2.0 * (h(0) + h(1));
      if (fabs(dg) < 1e-15) ok = false;
      else V.at(T_SPC, 1) = rhs(0) / dg;
    } else {
      // solve_thomas (thomas_solver.hpp:86-198) on rows j = 0..m-1:
      // lower h[j], diagonal 2(h[j] + h[j+1]), upper h[j+1].
      const double dg0 = 2.0 * (h(0) + h(1));
      if (fabs(dg0) < 1e-15) ok = false;
      double cp = h(1) / dg0, dp = rhs(0) / dg0;
      V.at(A_CP, 0) = cp;
      V.at(A_D, 0) = dp;
      for (int j = 1; j < m - 1 && ok; ++j) {
        const double lower = h(j);
        const double denom = fma(-lower, cp, 2.0 * (h(j) + h(j + 1)));
        if (fabs(denom) < 1e-15) { ok = false; break; }
        const double inv = 1.0 / denom;
        cp = h(j + 1) * inv;
        dp = fma(-lower, dp, rhs(j)) * inv;
        V.at(A_CP, j) = cp;
        V.at(A_D, j) = dp;
      }
      if (ok) {
        const int j = m - 1;
        const double lower = h(j);
        const double denom = fma(-lower, cp, 2.0 * (h(j) + h(j + 1)));
        if (fabs(denom) < 1e-15) ok = false;
        else {
          double s = fma(-lower, dp, rhs(j)) / denom;
          V.at(T_SPC, m) = s;
          for (int jj = m - 1; jj > 0; --jj) {
            s = fma(-V.at(A_CP, jj - 1), s, V.at(A_D, jj - 1));
            V.at(T_SPC, jj) = s;
          }
        }
      }
    }
    if (ok) {
      const double x_lo = L.x(0), x_hi = L.x(n - 1);
      for (int i = 0; i < n; ++i) {
        const double sk = exp(L.x(i));
        const double adj = sk - d;
        double u;
        if (adj > 1e-10) {
          const double xs = log(adj);
          if (xs < x_lo) {
            u = fallback;
          } else {
            const double xe = (x_hi < xs) ? x_hi : xs;
            const int iv = find_interval(L.X, n, xe);
            const double hi = h(iv);
            const double ci = V.at(T_SPC, iv), ci1 = V.at(T_SPC, iv + 1);
            const double bb = (y(iv + 1) - y(iv)) / hi - hi * (2.0 * ci + ci1) / 3.0;
            const double dd = (ci1 - ci) / (3.0 * hi);
            const double dx = xe - L.x(iv);
            u = y(iv) + bb * dx + ci * (dx * dx) + dd * (dx * dx * dx);
          }
        } else {
          u = fallback;
        }
        V.at(A_G, i) = u;
      }
    }
  }
  V.at(A_G, 0) = L.bcl;
  V.at(A_G, n - 1) = L.bcr(tau);
  for (int i = 0; i < n; ++i) V.at(A_G, i) = dmax_ref(V.at(A_G, i), V.at(A_PSI, i));
}

}  // namespace

// One warp per tile; lanes k >= mc.tv_first of the tiles [t_begin, ntiles).
__global__ void __launch_bounds__(128) march_tv_kernel(
    const TileDev* __restrict__ tiles, int t_begin, int ntiles, const OptDev* __restrict__ opts,
    const TvDev* __restrict__ tvs, const double* __restrict__ tv_tp,
    const double* __restrict__ tv_curve, const double* __restrict__ tv_ev,
    const double* __restrict__ xs, double* __restrict__ pool, int32_t* __restrict__ mode,
    int32_t* __restrict__ status, MarchConst mc) {
  const int lane = threadIdx.x & (kTile - 1);
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) / kTile;
  const int nwarps = (gridDim.x * blockDim.x) / kTile;
  for (int tile = t_begin + warp; tile < ntiles; tile += nwarps) {
    const TileDev td = tiles[tile];
    const int k = td.first + lane;
    if (lane >= td.count || k < mc.tv_first || (mc.active && !mc.active[k])) continue;
    const OptDev o = opts[k];
    const TvDev tv = tvs[k - mc.tv_first];
    Lane L;
    L.V = TileView{pool + td.off + lane, td.nx};
    L.X = xs + td.xoff + lane;
    L.n = o.n;
    L.put = o.is_put != 0;
    const double sigma = mc.sigma ? mc.sigma[k] : o.sigma;
    L.hss = 0.5 * sigma * sigma;
    L.q = o.q;
    L.bcl = o.bc_left;
    L.exp_xr = o.exp_xr;
    L.T = tv.T;
    L.r_const = tv.r;
    L.curve = Curve{tv_curve + 2 * static_cast<size_t>(tv.curve_off), tv.n_curve};
    tv_setup(L);
    mode[k] = L.uniform ? 2 : 0;
    const int nt = o.nt;
    const double* tp = tv.tp_off >= 0 ? tv_tp + tv.tp_off : nullptr;
    const double dt_avg = o.dt;
    auto tpt = [&](int i) { return tp ? tp[i] : static_cast<double>(i) * dt_avg; };
    auto dt_at = [&](int s) { return tp ? tp[s + 1] - tp[s] : dt_avg; };
    const double* ev = tv_ev + 2 * static_cast<size_t>(tv.ev_off);
    const double fallback = L.put ? 1.0 : 0.0;
    int e = 0;
    auto events = [&](double t_old, double t_new) {
      while (e < tv.n_ev) {
        const double tau = ev[2 * e];
        if (tau <= t_old) {
          ++e;
          continue;
        }
        if (tau > t_new) break;
        tv_dividend(L, tau, ev[2 * e + 1], fallback);
        ++e;
      }
    };
    int32_t st = kStatusOk;
    double t = tpt(0);
    int step = 0;
    if (mc.rannacher && nt > 0) {
      const double dt = dt_at(0);
      const double t_old = t, t_next = t + dt;
      const double half = 0.5 * dt;
      const double t_mid = t + half;
      if (!tv_stage<kEuler>(L, t_mid, half, 0.0, 0.0, 0.0)) st = kStatusSolver;
      if (st == kStatusOk) events(t_old, t_mid);
      if (st == kStatusOk && !tv_stage<kEuler>(L, t_next, half, 0.0, 0.0, 0.0)) st = kStatusSolver;
      if (st == kStatusOk) events(t_mid, t_next);
      t = tpt(1);
      step = 1;
    }
    for (; step < nt && st == kStatusOk; ++step) {
      const double t_old = t;
      const double dt = dt_at(step);
      const double t_next = tpt(step + 1);
      const double t_s1 = __dadd_rn(t, __dmul_rn(mc.gamma, dt));
      const double w1 = mc.gamma * dt / 2.0;
      const double w2 = (1.0 - mc.gamma) * dt / (2.0 - mc.gamma);
      if (!tv_stage<kTrap>(L, t_s1, w1, L.rate(t), 0.0, 0.0)) {
        st = kStatusSolver;
        break;
      }
      if (!tv_stage<kBdf2>(L, t_next, w2, 0.0, mc.alpha, mc.beta)) {
        st = kStatusSolver;
        break;
      }
      events(t_old, t_next);
      t = t_next;
    }
    // The result functionals read the final state from A_G and the previous
    // one from A_U, swapped after a Rannacher-only solve (outputs_kernel).
    if (st == kStatusOk && mc.rannacher && nt == 1) {
      for (int i = 0; i < L.n; ++i) {
        const double a = L.V.at(A_G, i);
        L.V.at(A_G, i) = L.V.at(A_U, i);
        L.V.at(A_U, i) = a;
      }
    }
    status[k] = st;
  }
}

}  // namespace mgpu
