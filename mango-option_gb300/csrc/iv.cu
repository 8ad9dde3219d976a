// iv.cu -- batched FDM implied volatility on the GPU.
//
// Restates IVSolver::solve / solve_brent (src/option/iv_solver.cpp:133-242)
// with brent_find_root (src/math/root_finding.hpp:145-302) as a per-quote
// state machine on the device.  Every quote keeps its own fixed grid; each
// evaluation re-prices the quotes still iterating at their trial
// volatilities with the same setup / march / value kernels as batched
// pricing, then one thread per quote consumes the objective values and
// proposes the next trial points.
//
// Two root finders share that pipeline:
//   MANGO_GPU_IV_BRENT   the reference's Brent, iterate for iterate (one
//                        trial point per quote per evaluation);
//   MANGO_GPU_IV_SECANT  starts at the Black-Scholes implied volatility of
//                        the quote, steps along the Black-Scholes vega, then
//                        by secant, inside the bracket seen so far.  While
//                        many quotes are iterating each gets one trial point
//                        per evaluation; once few are left, each gets k
//                        points (k = the resident march lanes / quotes
//                        left, at most 32): the secant point, points around
//                        it, a k-section of the bracket and, while a side of
//                        the bracket is unverified, Brent's bracket end
//                        there.  A round of one tile per resident warp costs
//                        about as long as a lone warp's march (per-warp
//                        latency, not throughput, sets it), so the extra
//                        points are nearly free and cut the number of
//                        evaluations the last quotes need.  Once a sign
//                        change of V - P is seen the search keeps a
//                        sign-change bracket, so it converges even where V
//                        is not monotone in the volatility.  Quotes that go
//                        non-finite, or find no sign change within
//                        kFastMaxEvals evaluations, are re-solved by Brent.
// Both stop on the reference's test |V(sigma) - P| < tol (or a bracket
// narrower than tol).
//
// Each evaluation packs the trial points still to price into tiles of 32 in
// sorted order (one gather of grids and parameters on the device), so
// finished quotes never occupy warps.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "brent.cuh"
#include "engine.hpp"
#include "march_tan.cuh"
#include "wmarch.cuh"

namespace mgpu {

using namespace brentdev;

// Evaluations of the fast root finder before a quote without a sign change
// is handed to Brent, and the cap for a quote inside a sign-change bracket
// (which at least halves every second evaluation).
constexpr int kFastMaxEvals = 12;
constexpr int kFastMaxBracketEvals = 60;
// Trial points per quote and evaluation, at most.
constexpr int kMaxPts = 32;
// IVSolver::solve_brent lower bracket (iv_solver.cpp:150).
constexpr double kVolLower = 0.01;
// Volatility-space tolerance of quotes the Newton path hands to the
// k-section finder: a sign-change bracket this narrow settles them.
constexpr double kVolTol = 1e-7;
// A sign-change bracket at most this wide: its secant stands for the local
// slope in the settle test of a Newton hand-over.
constexpr double kNarrowBracket = 1e-3;

// Fast root-finder state of one quote.  Until a sign change of f has been
// seen, [lo, hi] steers the search assuming f rises with the volatility;
// from then on [bl, br] always holds a sign change (f(bl) f(br) < 0), so
// the search converges whether or not f is monotone.
struct FastDev {
  double lo, hi;   // steering bounds: f(lo) < 0 (seen bit 0), f(hi) > 0 (seen bit 1)
  double flo, fhi;
  double bl, br;   // sign-change bracket, when has_br
  double fl, fr;
  double xa, fa;   // best point so far (smallest |f|), f signed
  double xb, fb;   // second best point
  double e0, e1;   // f at Brent's bracket ends 0.01 and upper, when evaluated
  double guess;    // Black-Scholes implied volatility of the price
  double width;    // bracket width before the last evaluation
  double ftol;     // > 0: settle on |f| < ftol or a bracket narrower than kVolTol
                   // (a quote Newton handed over); 0: the call's price tolerance
  int32_t iter;    // evaluations consumed
  int32_t seen;
  int32_t ends;    // bit 0: f(0.01) evaluated; bit 1: f(upper) evaluated
  int32_t has_br;
};

// Newton on a coarse grid, then the secant on the quote's own grid.
//   level 0: kCoarseEvals Newton steps with the exact discrete vega (the
//            volatility tangent of the march) on a coarse grid of the same
//            kind (2/5 of the space points, an eighth of the time steps)
//            from the Black-Scholes implied volatility; the two vegas give
//            the curvature d(vega)/d(sigma);
//   level 1: value-only evaluations on the quote's own grid: a first step
//            from the coarse root with the coarse vega (and its curvature),
//            then secant steps, corrected by the curvature of the parabola
//            through the last three values.  A quote settles once the
//            secant step through its last two own-grid values is at most
//            kSecantAccept, at that step's end point.
struct NewtonDev {
  double x;        // point evaluated this round
  double lo, hi;   // f(lo) < 0 < f(hi) where seen, else the Brent bracket ends
  double flo, fhi; // f there (seen bits)
  double kc;       // coarse curvature estimate d(vega)/d(sigma)
  double xp, vp;   // previous point on this level; its vega on the coarse level
  double x0;       // starting point (Black-Scholes implied volatility)
  double xb, fb;   // own-grid point with the smallest |f|
  double vs;       // coarse vega carried to the first own-grid point
  double sec;      // slope of the secant through the last two own-grid values
  double fp;       // f at xp (own grid)
  double xpp, fpp; // the own-grid point before xp
  int32_t has_pp;
  int32_t level;   // 0 coarse, 1 own grid
  int32_t it;      // evaluations on this level
  int32_t total;   // evaluations overall
  int32_t has_prev;
  int32_t seen;    // bit 0: f(lo) < 0 evaluated, bit 1: f(hi) > 0 evaluated
};

// Per-quote root-finder state.
struct IvDev {
  BrentDev br;
  FastDev fs;
  NewtonDev nw;
  int32_t mode;  // 0 fast, 1 Brent, 2 finished, 3 Newton
  int32_t pad;
};

// Newton schedule: evaluations on the coarse grid, evaluations on the
// quote's own grid before a hand-over to the k-section finder, and the
// acceptance test on the own grid.  A secant step of at most kSecantAccept
// through two own-grid values leaves an error of that step times the
// relative change of the slope over it: below 1e-7 in volatility even where
// the discrete objective's slope jumps by a few per cent as grid rows enter
// or leave the exercise region.  Larger unverified steps (a Newton step from
// a single evaluation) were measured to miss by up to 2e-6 across such jumps.
constexpr int kCoarseEvals = 2;
constexpr int kOwnEvals = 6;
constexpr double kSecantAccept = 3e-6;
// Below this vega (per unit volatility, relative to max(1, price)) the
// objective is flat: the volatility is not determined by the price, and the
// reference's price test |V - P| < tol settles the quote.
constexpr double kFlatVega = 1e-7;

// Final result of one quote.
struct IvOut {
  double root, ferr;
  int32_t iter, code;
  double vega;  // Newton-settled quotes: the slope of the last own-grid secant; else NaN
};

namespace {

// ------------------------------------------------------ fast finder --

// Black-Scholes price with continuous dividend yield (closed form).
__device__ double bs_price(bool put, double S, double K, double T, double r, double q,
                           double sig) {
  const double st = sig * sqrt(T);
  const double d1 = (log(S / K) + (r - q + 0.5 * sig * sig) * T) / st;
  const double d2 = d1 - st;
  const double dfq = exp(-q * T), dfr = exp(-r * T);
  const double h = 0.7071067811865476;  // 1/sqrt(2): N(z) = erfc(-z/sqrt(2))/2
  if (put) return K * dfr * 0.5 * erfc(d2 * h) - S * dfq * 0.5 * erfc(d1 * h);
  return S * dfq * 0.5 * erfc(-d1 * h) - K * dfr * 0.5 * erfc(-d2 * h);
}

// Black-Scholes vega (same for puts and calls).
__device__ double bs_vega(double S, double K, double T, double r, double q, double sig) {
  const double st = sqrt(T);
  const double d1 = (log(S / K) + (r - q + 0.5 * sig * sig) * T) / (sig * st);
  return S * exp(-q * T) * st * exp(-0.5 * d1 * d1) * 0.3989422804014327;  // 1/sqrt(2 pi)
}

// European implied volatility of the quote's price inside [lo, hi] by
// bisection-safeguarded Newton; only a starting point (the American price
// is what gets matched).  A price outside the European range on [lo, hi]
// starts at the nearer end.
__device__ double european_iv_guess(bool put, double S, double K, double T, double r, double q,
                                    double P, double lo, double hi) {
  double a = lo, b = hi;
  if (!(bs_price(put, S, K, T, r, q, a) - P < 0.0)) return lo;
  if (!(bs_price(put, S, K, T, r, q, b) - P > 0.0)) return hi;
  double x = fmin(fmax(0.3, a), b);
  for (int it = 0; it < 40; ++it) {
    const double f = bs_price(put, S, K, T, r, q, x) - P;
    if (fabs(f) < 1e-12 * fmax(P, 1.0)) break;
    if (f > 0.0) b = x; else a = x;
    const double v = bs_vega(S, K, T, r, q, x);
    double xn = v > 0.0 ? x - f / v : 0.5 * (a + b);
    if (!(xn > a && xn < b)) xn = 0.5 * (a + b);
    const bool small = fabs(xn - x) < 1e-12;
    x = xn;
    if (small) break;
  }
  return x;
}

constexpr int kFastGo = 0, kFastSettled = 1, kFastBracket = 2, kFastHandOver = 3;

// Consume the n objective values f[j] at sig[j].  Settled when a point has
// |f| < tol (the Brent stopping test, root_finding.hpp:210-218) or the
// sign-change bracket is narrower than tol.  With f evaluated at both of
// Brent's bracket ends and no sign change anywhere, the quote fails as
// Brent's does (root_finding.hpp:176-185).
__device__ int fast_consume(FastDev& s, const double* sig, const double* f, int n, double upper,
                            double tol) {
  s.iter += 1;
  s.width = s.has_br ? s.br - s.bl : s.hi - s.lo;
  for (int j = 0; j < n; ++j)
    if (!isfinite(f[j])) return kFastHandOver;
  // A quote Newton handed over whose objective is flat within the call's
  // tolerance: two points (of this round, or one of them the best point so
  // far) with |f| < tol and a secant slope not above kFlatVega, where the
  // volatility is not determined by the price (the spot node locked to the
  // payoff over a range of volatilities).  It settles on the reference's
  // test, as Newton's own flat stop does, at its best point.
  bool flat = false;
  if (s.ftol > 0.0) {
    for (int j = 0; j < n && !flat; ++j) {
      if (!(fabs(f[j]) < tol)) continue;
      if (fabs(s.fa) < tol && sig[j] != s.xa &&
          (f[j] - s.fa) / (sig[j] - s.xa) <= kFlatVega)
        flat = true;
      for (int l = j + 1; l < n && !flat; ++l)
        if (fabs(f[l]) < tol && sig[l] != sig[j] && (f[l] - f[j]) / (sig[l] - sig[j]) <= kFlatVega)
          flat = true;
    }
  }
  for (int j = 0; j < n; ++j) {
    const double x = sig[j], fj = f[j];
    if (fabs(fj) < fabs(s.fa)) {
      s.xb = s.xa;
      s.fb = s.fa;
      s.xa = x;
      s.fa = fj;
    } else if (fabs(fj) < fabs(s.fb) && x != s.xa) {
      s.xb = x;
      s.fb = fj;
    }
    if (x == kVolLower) {
      s.ends |= 1;
      s.e0 = fj;
    }
    if (x == upper) {
      s.ends |= 2;
      s.e1 = fj;
    }
    if (fj < 0.0 && (!(s.seen & 1) || x > s.lo)) {
      s.lo = x;
      s.flo = fj;
      s.seen |= 1;
    } else if (fj > 0.0 && (!(s.seen & 2) || x < s.hi)) {
      s.hi = x;
      s.fhi = fj;
      s.seen |= 2;
    }
  }
  double ptol = s.ftol > 0.0 ? s.ftol : tol;
  const double btol = s.ftol > 0.0 ? kVolTol : tol;
  if (s.ftol > 0.0 && s.has_br && s.fr > s.fl) {
    // a Newton hand-over settles within kVolTol along the bracket's own
    // slope: when that is the smaller one while the bracket is wide, and
    // alone once it is narrower than kNarrowBracket
    const double sb = kVolTol * (s.fr - s.fl) / (s.br - s.bl);
    ptol = (s.br - s.bl <= kNarrowBracket) ? sb : fmin(ptol, sb);
  }
  if (fabs(s.fa) < ptol || flat) return kFastSettled;
  if (!s.has_br && s.seen == 3) {
    s.has_br = 1;
    if (s.lo < s.hi) {
      s.bl = s.lo, s.fl = s.flo, s.br = s.hi, s.fr = s.fhi;
    } else {
      s.bl = s.hi, s.fl = s.fhi, s.br = s.lo, s.fr = s.flo;
    }
  }
  if (s.has_br) {
    // Narrow to the first sign change along bl < points inside < br.
    double px[kMaxPts], pf[kMaxPts];
    int m = 0;
    for (int j = 0; j < n; ++j)
      if (sig[j] > s.bl && sig[j] < s.br) {
        int i = m++;
        while (i > 0 && px[i - 1] > sig[j]) {
          px[i] = px[i - 1];
          pf[i] = pf[i - 1];
          --i;
        }
        px[i] = sig[j];
        pf[i] = f[j];
      }
    double xl = s.bl, fl = s.fl;
    for (int i = 0; i < m; ++i) {
      if ((fl < 0.0) != (pf[i] < 0.0)) {
        s.br = px[i];
        s.fr = pf[i];
        break;
      }
      xl = px[i];
      fl = pf[i];
    }
    s.bl = xl;
    s.fl = fl;
    if (s.br - s.bl < btol) return kFastSettled;
  } else if (s.ends == 3) {
    return kFastBracket;
  }
  if (s.iter >= (s.has_br ? kFastMaxBracketEvals : kFastMaxEvals)) return kFastHandOver;
  return kFastGo;
}

// Up to k next trial points into pts (distinct); returns how many.
__device__ int fast_propose(const FastDev& s, const OptDev& o, double T, double upper, int k,
                            double* pts) {
  int n = 0;
  auto add = [&](double x) {
    if (n >= k || !(x >= kVolLower && x <= upper)) return;
    for (int j = 0; j < n; ++j)
      if (fabs(pts[j] - x) <= 1e-14 * x) return;
    pts[n++] = x;
  };
  const double lo = s.has_br ? s.bl : s.lo;
  // A Newton hand-over that has only seen f < 0 searches upward in ranges
  // of a factor 4 (trial volatilities far above the grid's march slowly, and
  // its root is usually close): Brent's upper end only once the range
  // reaches it.
  const bool climb = s.ftol > 0.0 && !s.has_br && s.seen == 1;
  const double hi = s.has_br ? s.br : (climb ? fmin(s.hi, 4.0 * s.lo) : s.hi);
  auto inside = [&](double x) { return x > lo && x < hi; };
  // centre: the secant through the two best points, a Black-Scholes-vega
  // Newton step from a lone point, or the starting guess; inside a
  // sign-change bracket the false-position point when the secant leaves
  // it, and the midpoint when the last evaluation did not halve it
  double c, w;
  if (s.iter == 0) {
    c = s.guess;
    w = 0.1 * c;
  } else {
    if (isfinite(s.fb) && s.fb != s.fa) {
      c = s.xa - s.fa * (s.xa - s.xb) / (s.fa - s.fb);
    } else {
      c = s.xa - s.fa / bs_vega(o.spot, o.strike, T, o.r, o.q, s.xa);
    }
    if (s.has_br) {
      if (!inside(c)) c = s.bl - s.fl * (s.br - s.bl) / (s.fr - s.fl);
      if (!inside(c) || (k == 1 && s.br - s.bl > 0.5 * s.width)) c = 0.5 * (s.bl + s.br);
    } else if (!inside(c)) {
      c = 0.5 * (lo + hi);
    }
    w = 2.0 * fabs(c - s.xa);
  }
  add(c);
  if (k >= 3 && !s.has_br) {
    // Brent's bracket ends (f at both, without a sign change, fails the
    // quote as Brent fails it).  A Newton hand-over has seen one sign
    // already: it tries the end that may show the other, and the far end
    // only once that one has not (trial volatilities far above the grid's
    // march slowly).
    const bool nh = s.ftol > 0.0;
    if (!(s.ends & 1) && (!nh || !(s.seen & 1) || (s.ends & 2))) add(kVolLower);
    if (!(s.ends & 2) && (!nh || !(s.seen & 2) || (s.ends & 1)) && !(climb && hi < upper)) add(upper);
  }
  const int rest = k - n;
  const int near = rest / 2, spread = rest - near;
  for (int j = 1; j <= near; ++j) {
    const double off = w * static_cast<double>((j + 1) / 2) / static_cast<double>((near + 1) / 2);
    const double x = (j & 1) ? c + off : c - off;
    if (inside(x)) add(x);
  }
  // evenly over [lo, hi]; for a Newton hand-over whose bracket spans more
  // than a factor 4, evenly in log volatility
  const bool geometric = s.ftol > 0.0 && hi > 4.0 * lo;
  for (int j = 1; j <= spread; ++j) {
    const double t = static_cast<double>(j) / static_cast<double>(spread + 1);
    const double x = geometric ? lo * pow(hi / lo, t) : lo + (hi - lo) * t;
    if (inside(x)) add(x);
  }
  return n;
}

// Objective at working slot k: V(sigma) - P (iv_solver.cpp:48-119); a failed
// march gives NaN, as the reference's objective does.
__device__ __forceinline__ double objective(const double* out4, const int32_t* mstatus, int k,
                                            double price) {
  return mstatus[k] == kStatusOk ? out4[4 * static_cast<size_t>(k)] - price : qnan();
}

// Working sets of an evaluation round: the coarse grids with the volatility
// tangent (Newton's first evaluations) and the quotes' own grids without it
// (Newton's later evaluations, Brent, the secant, time-varying quotes).
constexpr int32_t kLevelCoarse = 0, kLevelPlain = 1, kLevels = 2;
// Quotes left at or below which a round re-orders its working set.
constexpr int64_t kTailQuotes = 65536;

// Newton on f = V - P at s.x; v = dV/dsigma on the coarse level (the
// evaluation carried the tangent).  Coarse level: exactly kCoarseEvals
// evaluations (all quotes reach their own grid in the same round), the
// curvature from the last two.  Own grid: value-only steps as described at
// NewtonDev.  Returns 0 to go on (s.x is the next point, *level its working
// set), 1 when settled at *root (*vega: the last secant's slope, or NaN),
// 2 to hand the quote over.
__device__ int newton_consume(NewtonDev& s, double f, double v, double upper, double tol,
                              double* root, double* vega, int32_t* level) {
  s.total += 1;
  s.it += 1;
  const double x = s.x;
  *vega = qnan();
  if (s.level == 0) {
    const bool good = isfinite(f) && isfinite(v) && v > 0.0;
    if (good) {
      if (s.has_prev && x != s.xp) s.kc = (v - s.vp) / (x - s.xp);
      s.xp = x;
      s.vp = v;
      s.has_prev = 1;
      s.x = fmin(fmax(x - f / v, kVolLower), upper);
    } else {
      s.x = s.x0;
    }
    if (s.it >= kCoarseEvals) {
      s.vs = s.has_prev ? s.vp + s.kc * (s.x - s.xp) : qnan();
      s.level = 1;
      s.it = 0;
      s.has_prev = 0;
    }
    *level = s.level == 0 ? kLevelCoarse : kLevelPlain;
    return 0;
  }
  *level = kLevelPlain;
  if (!isfinite(f)) return 2;
  if (f < 0.0 && (!(s.seen & 1) || x > s.lo)) {
    s.lo = x;
    s.flo = f;
    s.seen |= 1;
  } else if (f > 0.0 && (!(s.seen & 2) || x < s.hi)) {
    s.hi = x;
    s.fhi = f;
    s.seen |= 2;
  }
  if (!(fabs(f) >= fabs(s.fb))) {
    s.xb = x;
    s.fb = f;
  }
  if (f == 0.0) {
    *root = x;
    *vega = s.sec;
    return 1;
  }
  double slope, kk = s.kc;
  if (!s.has_prev) {
    slope = s.vs;  // first own-grid point: the coarse vega carried there
    if (!(slope > 0.0)) return 2;
  } else {
    if (x == s.xp) return 2;
    const double sec = (f - s.fp) / (x - s.xp);
    s.sec = sec;
    const double flat = kFlatVega * fmax(1.0, fabs(f) + fabs(s.fb));
    if (!(sec > flat)) {
      if (fabs(f) < tol) {  // flat objective: the reference's stopping test
        *root = x;
        return 1;
      }
      return 2;
    }
    const double d = -f / sec;
    const double xs = x + d;
    if (fabs(d) <= kSecantAccept && xs >= kVolLower && xs <= upper) {
      *root = xs;
      *vega = sec;
      return 1;
    }
    // the parabola through the last three values; with two, the coarse
    // curvature
    if (s.has_pp && x != s.xpp) kk = 2.0 * (sec - (s.fp - s.fpp) / (s.xp - s.xpp)) / (x - s.xpp);
    slope = sec + 0.5 * kk * (x - s.xp);
    if (!(slope > 0.0)) return 2;
  }
  if (s.it >= kOwnEvals || (s.seen == 3 && !(s.lo < s.hi))) return 2;
  if (s.has_prev) {
    s.xpp = s.xp;
    s.fpp = s.fp;
    s.has_pp = 1;
  }
  s.xp = x;
  s.fp = f;
  s.has_prev = 1;
  // second-order step on f + slope d + kk d^2 / 2 = 0 (fixed point, where
  // the correction is small against the step)
  const double d = -f / slope;
  double dh = d;
  if (fabs(kk * d / slope) < 0.5)
    for (int k = 0; k < 3; ++k) dh = -(f + 0.5 * kk * dh * dh) / slope;
  double xn = fmin(fmax(x + dh, kVolLower), upper);
  if (s.seen == 3 && !(xn > s.lo && xn < s.hi)) xn = 0.5 * (s.lo + s.hi);
  s.x = xn;
  return 0;
}

// Hand a quote Newton did not settle to the secant / k-section finder on
// the plain working set, seeded with what Newton learned: the bracket ends it
// evaluated and its best point.
__device__ void newton_to_fast(const NewtonDev& n, FastDev& s, double upper) {
  s = FastDev{};
  s.lo = (n.seen & 1) ? n.lo : kVolLower;
  s.hi = (n.seen & 2) ? n.hi : upper;
  s.flo = n.flo;
  s.fhi = n.fhi;
  s.seen = n.seen;
  s.xa = n.xb;
  s.fa = isfinite(n.fb) ? n.fb : pinf();
  s.xb = qnan();
  s.fb = pinf();
  s.e0 = s.e1 = qnan();
  s.guess = isfinite(n.xb) ? n.xb : n.x0;
  s.iter = 1;  // the first proposal uses the best point, not the guess
  // settle at |f| < 1e-7 vol times the slope: the own grid's last secant,
  // else the smaller of the coarse vega and the vega floor 1e-4 (a quote
  // whose slope is unknown settles on its bracket instead)
  const double slope = n.sec > 0.0 ? n.sec : (n.vs > 0.0 ? fmin(n.vs, 1e-4) : 1e-4);
  s.ftol = kVolTol * slope;
  if (s.seen == 3) {
    s.has_br = 1;
    if (s.lo < s.hi) {
      s.bl = s.lo, s.fl = s.flo, s.br = s.hi, s.fr = s.fhi;
    } else {
      s.bl = s.hi, s.fl = s.fhi, s.br = s.lo, s.fr = s.flo;
    }
  }
}

}  // namespace

// First trial points of every sorted quote: the Black-Scholes implied vol
// and up to k - 1 more (fast), or the lower bracket 0.01 (Brent).
__global__ void iv_init_kernel(int m, int32_t method, int k, int tv_first,
                               const OptDev* __restrict__ opts, const double* __restrict__ mat,
                               const double* __restrict__ price, const double* __restrict__ upper,
                               IvDev* __restrict__ S, IvOut* __restrict__ R,
                               double* __restrict__ next_sig, int32_t* __restrict__ npts,
                               int32_t* __restrict__ lev) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  R[q] = IvOut{qnan(), qnan(), 0, kIvNumerical, qnan()};
  IvDev st{};
  double* pts = next_sig + static_cast<size_t>(q) * kMaxPts;
  lev[q] = kLevelPlain;
  if (method == MANGO_GPU_IV_NEWTON && q < tv_first) {
    const OptDev o = opts[q];
    NewtonDev& s = st.nw;
    s.lo = kVolLower;
    s.hi = upper[q];
    s.x0 = european_iv_guess(o.is_put != 0, o.spot, o.strike, mat[q], o.r, o.q, price[q], s.lo,
                             s.hi);
    s.x = s.x0;
    s.xb = qnan();
    s.fb = pinf();
    s.vs = s.sec = s.fp = qnan();
    st.mode = 3;
    pts[0] = s.x;
    npts[q] = 1;
    lev[q] = kLevelCoarse;
  } else if (method == MANGO_GPU_IV_SECANT || method == MANGO_GPU_IV_NEWTON) {
    const OptDev o = opts[q];
    FastDev& s = st.fs;
    s.lo = kVolLower;
    s.hi = upper[q];
    s.guess = european_iv_guess(o.is_put != 0, o.spot, o.strike, mat[q], o.r, o.q, price[q], s.lo,
                                s.hi);
    s.xa = s.xb = qnan();
    s.fa = s.fb = pinf();
    s.e0 = s.e1 = qnan();
    st.mode = 0;
    npts[q] = fast_propose(s, o, mat[q], s.hi, k, pts);
  } else {
    brent_start(st.br, kVolLower, upper[q]);
    st.mode = 1;
    pts[0] = st.br.a;
    npts[q] = 1;
  }
  S[q] = st;
}

// Consume the objective values of quote qlist[i] (slots qbase[i] ..
// qbase[i] + npts - 1) and propose its next trial points (k at most for
// the fast finder); npts[q] = 0 once the quote is finished.
__global__ void iv_step_kernel(int nq, const int32_t* __restrict__ qlist,
                               const int32_t* __restrict__ qbase, int k, IvDev* __restrict__ S,
                               IvOut* __restrict__ R, const OptDev* __restrict__ opts,
                               const double* __restrict__ mat, const double* __restrict__ upper,
                               const double* __restrict__ out4, const int32_t* __restrict__ mstatus,
                               const double* __restrict__ sigma_w, const double* __restrict__ price,
                               double* __restrict__ next_sig, int32_t* __restrict__ npts, double tol,
                               int max_iter, int trace, int has_vega, int32_t* __restrict__ lev) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const int q = qlist[i];
  const int base = qbase[i];
  const int n = min(npts[q], kMaxPts);
  IvDev st = S[q];
  double* pts = next_sig + static_cast<size_t>(q) * kMaxPts;
  const double P = price[q];
  int next_n = 0;
  if (st.mode == 0) {
    double sg[kMaxPts], fv[kMaxPts];
    for (int j = 0; j < n; ++j) {
      sg[j] = sigma_w[base + j];
      fv[j] = objective(out4, mstatus, base + j, P);
    }
    const int r = fast_consume(st.fs, sg, fv, n, upper[q], tol);
    if (trace && st.fs.ftol > 0.0)
      printf("iv k-section orig=%d iter=%d r=%d n=%d br=%d [%.17g, %.17g] lo=%.17g hi=%.17g "
             "seen=%d xa=%.17g fa=%.6e xb=%.17g fb=%.6e ftol=%.3e\n",
             opts[q].orig, st.fs.iter, r, n, st.fs.has_br, st.fs.bl, st.fs.br, st.fs.lo, st.fs.hi,
             st.fs.seen, st.fs.xa, st.fs.fa, st.fs.xb, st.fs.fb, st.fs.ftol);
    if (r == kFastGo) {
      next_n = fast_propose(st.fs, opts[q], mat[q], upper[q], k, pts);
    } else if (r == kFastSettled) {
      R[q] = IvOut{st.fs.xa, fabs(st.fs.fa), st.fs.iter, kIvOk, qnan()};
      st.mode = 2;
    } else if (r == kFastBracket) {
      R[q] = IvOut{qnan(), fmin(fabs(st.fs.e0), fabs(st.fs.e1)), 0, kIvBracket, qnan()};
      st.mode = 2;
    } else {
      if (trace)
        printf("iv hand-over q=%d iter=%d lo=%.17g hi=%.17g seen=%d ends=%d bracket=%d [%.17g, %.17g] "
               "xa=%.17g fa=%.6e xb=%.17g fb=%.6e guess=%.6g n=%d\n",
               q, st.fs.iter, st.fs.lo, st.fs.hi, st.fs.seen, st.fs.ends, st.fs.has_br, st.fs.bl,
               st.fs.br, st.fs.xa, st.fs.fa, st.fs.xb, st.fs.fb, st.fs.guess, n);
      brent_start(st.br, kVolLower, upper[q]);
      st.mode = 1;
      pts[0] = st.br.a;
      next_n = 1;
    }
  } else if (st.mode == 3) {
    const double f = objective(out4, mstatus, base, P);
    const double v = (has_vega && mstatus[base] == kStatusOk)
                         ? out4[4 * static_cast<size_t>(base) + 3] : qnan();
    double root = qnan(), vega = qnan();
    int32_t level = kLevelPlain;
    const int r = newton_consume(st.nw, f, v, upper[q], tol, &root, &vega, &level);
    if (r == 0) {
      pts[0] = st.nw.x;
      next_n = 1;
      lev[q] = level;
    } else if (r == 1) {
      R[q] = IvOut{root, fabs(f), st.nw.total, kIvOk, vega};
      st.mode = 2;
    } else {
      if (trace)
        printf("iv newton hand-over orig=%d total=%d x=%.17g f=%.6e seen=%d lo=%.17g hi=%.17g "
               "flo=%.6e fhi=%.6e xb=%.17g fb=%.6e sec=%.6e vs=%.6e\n",
               opts[q].orig, st.nw.total, st.nw.x, f, st.nw.seen, st.nw.lo, st.nw.hi, st.nw.flo,
               st.nw.fhi, st.nw.xb, st.nw.fb, st.nw.sec, st.nw.vs);
      newton_to_fast(st.nw, st.fs, upper[q]);
      st.mode = 0;
      next_n = fast_propose(st.fs, opts[q], mat[q], upper[q], k, pts);
      lev[q] = kLevelPlain;
    }
  } else if (st.mode == 1) {
    double next = 0.0;
    if (brent_consume(st.br, objective(out4, mstatus, base, P), tol, max_iter, &next)) {
      pts[0] = next;
      next_n = 1;
    } else {
      R[q] = IvOut{st.br.root, st.br.ferr, st.br.iter, st.br.code, qnan()};
      st.mode = 2;
    }
  }
  npts[q] = next_n;
  S[q] = st;
}

// Gather the working set from the batch (sorted order, tile t holding
// sorted quotes [32 t, 32 t + 32)): slot k prices quote map[k] at its trial
// point pt[k].
__global__ void iv_gather_kernel(int mw, const int32_t* __restrict__ map,
                                 const int32_t* __restrict__ src_map,
                                 const int32_t* __restrict__ pt,
                                 const TileDev* __restrict__ src_tiles,
                                 const OptDev* __restrict__ src_opts,
                                 const double* __restrict__ src_xs,
                                 const TileDev* __restrict__ dst_tiles,
                                 OptDev* __restrict__ dst_opts, double* __restrict__ dst_xs,
                                 const double* __restrict__ next_sig,
                                 double* __restrict__ sigma_w, int32_t* __restrict__ active_w) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= mw) return;
  const int q = map[k];
  const int qs = src_map ? src_map[k] : q;  // the quote's index in the source batch
  const OptDev o = src_opts[qs];
  dst_opts[k] = o;
  const TileDev ts = src_tiles[qs / kTile];
  const TileDev td = dst_tiles[k / kTile];
  const double* src = src_xs + ts.xoff + (qs % kTile);
  double* dst = dst_xs + td.xoff + (k % kTile);
  for (int i = 0; i < td.nx; ++i)
    dst[static_cast<size_t>(i) * kTile] = src[static_cast<size_t>(min(i, o.n - 1)) * kTile];
  sigma_w[k] = next_sig[static_cast<size_t>(q) * kMaxPts + pt[k]];
  active_w[k] = 1;
}

// Schedule data of the working set's time-varying slots: slot j takes the
// per-option data of its quote (batch sorted index map[j], whose data sit
// at map[j] - tv_first_b); time points, curves and events stay in the
// batch's arrays.
__global__ void iv_gather_tv_kernel(int n, const int32_t* __restrict__ map, int tv_first_b,
                                    const TvDev* __restrict__ src, TvDev* __restrict__ dst) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < n) dst[j] = src[map[j] - tv_first_b];
}

// Status of an IV query before any solve, as the reference C ABI reports
// it: build_iv_query (src/ffi/mango_c_api.cpp:168-203) rejects a bad option
// type and non-finite rate or dividend yield with MANGO_ERR_VALIDATION; then
// validate_iv_query (src/option/option_spec.cpp:52-112) through
// validation_error_to_iv_error (src/option/iv_result.hpp:55-99) and
// map_iv_error (mango_c_api.cpp:124-141): bad spot / strike / maturity /
// non-positive price -> VALIDATION, negative dividend yield and a price
// outside [intrinsic, upper bound] -> ARBITRAGE.  Yield curves and discrete
// dividends are outside the engine's scope (VALIDATION).
int32_t iv_query_status(const MangoIvQuery& q, std::string* msg) {
  auto bad = [&](int32_t code, const char* m) {
    *msg = m;
    return code;
  };
  if (q.option_type != MANGO_PUT && q.option_type != MANGO_CALL)
    return bad(MANGO_ERR_VALIDATION, "invalid option type");
  {
    // build_rate / build_dividends, and the dividend rules of
    // validate_iv_query (src/option/option_spec.cpp:89-110)
    const std::string m = schedule_error(q.tenor_points, q.n_tenor_points, q.dividends, q.n_dividends,
                                         q.maturity);
    if (!m.empty()) {
      *msg = m;
      return MANGO_ERR_VALIDATION;
    }
  }
  if (!std::isfinite(q.dividend_yield)) return bad(MANGO_ERR_VALIDATION, "dividend_yield must be finite");
  if (q.n_tenor_points == 0 && !std::isfinite(q.rate_const))
    return bad(MANGO_ERR_VALIDATION, "rate must be finite");
  if (!(q.spot > 0.0) || !std::isfinite(q.spot)) return bad(MANGO_ERR_VALIDATION, "invalid spot");
  if (!(q.strike > 0.0) || !std::isfinite(q.strike)) return bad(MANGO_ERR_VALIDATION, "invalid strike");
  if (!(q.maturity > 0.0) || !std::isfinite(q.maturity))
    return bad(MANGO_ERR_VALIDATION, "invalid maturity");
  if (q.dividend_yield < 0.0) return bad(MANGO_ERR_ARBITRAGE, "invalid dividend yield");
  if (!std::isfinite(q.market_price) || q.market_price <= 0.0)
    return bad(MANGO_ERR_VALIDATION, "invalid market price");
  const bool put = q.option_type == MANGO_PUT;
  const double intrinsic = put ? std::max(q.strike - q.spot, 0.0) : std::max(q.spot - q.strike, 0.0);
  const double upper = put ? q.strike : q.spot;
  if (q.market_price < intrinsic) return bad(MANGO_ERR_ARBITRAGE, "market price below intrinsic value");
  if (q.market_price > upper) return bad(MANGO_ERR_ARBITRAGE, "market price above the upper bound");
  return MANGO_OK;
}

namespace {

using Clock = std::chrono::steady_clock;

double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// The trial points of one evaluation packed into tiles of 32 (sorted
// order), with the device buffers their marches use.  Quotes are indexed by
// their position in the batch b; their grids and parameters come from the
// batch src (b itself, or the coarse-grid batch of the Newton method, where
// smap maps b's sorted index to src's).  A tangent working set also carries
// the volatility tangent (march_tan.cu).
struct WorkSet {
  MangoGpuBatch* b = nullptr;
  MangoGpuBatch* src = nullptr;
  const std::vector<int32_t>* smap = nullptr;
  bool tangent = false;
  cudaStream_t st = nullptr;
  int64_t mw = 0;  // slots
  int32_t ntiles = 0;
  int64_t nq = 0;  // quotes
  int64_t pool_doubles = 0;
  std::vector<int32_t> map_h, src_h, pt_h, qlist_h, qbase_h;
  std::vector<TileDev> tiles_h;
  DevBuf d_tiles, d_opts, d_xs, d_map, d_src, d_pt, d_qlist, d_qbase, d_sigma, d_active, d_pool,
      d_flags, d_mode, d_status, d_out4, d_tv, d_tpool, d_wt, d_twarp, d_ho;
  // First slot of a time-varying quote (slots follow the batch order, where
  // those quotes come last), or INT32_MAX.
  int32_t tv_first = 0x7fffffff;

  // The context's buffers this set uses for the solve (swapped in by
  // borrow, back out on destruction), or null: released on destruction.
  DevBuf* home = nullptr;

  std::array<DevBuf*, kIvWorkBufs> bufs() {
    return {&d_tiles, &d_opts, &d_xs, &d_map, &d_src, &d_pt, &d_qlist, &d_qbase, &d_sigma,
            &d_active, &d_pool, &d_flags, &d_mode, &d_status, &d_out4, &d_tv, &d_tpool, &d_wt,
            &d_twarp, &d_ho};
  }
  void borrow(DevBuf* h) {
    home = h;
    const auto l = bufs();
    for (int i = 0; i < kIvWorkBufs; ++i) std::swap(*l[i], h[i]);
  }
  ~WorkSet() {
    const auto l = bufs();
    for (int i = 0; i < kIvWorkBufs; ++i) {
      if (home)
        std::swap(*l[i], home[i]);
      else
        l[i]->release();
    }
  }

  // Slots for the quotes in `active` (ascending) with npts[q] > 0.  The
  // host arrays must stay untouched until the stream has passed the copies.
  void pack(const std::vector<int32_t>& active, const int32_t* npts, const double* next_sig) {
    map_h.clear();
    src_h.clear();
    pt_h.clear();
    qlist_h.clear();
    qbase_h.clear();
    for (int32_t q : active) {
      const int c = std::min(npts[q], kMaxPts);
      if (c <= 0) continue;
      qlist_h.push_back(q);
      qbase_h.push_back(static_cast<int32_t>(map_h.size()));
      const int32_t qs = smap ? (*smap)[q] : q;
      for (int j = 0; j < c; ++j) {
        map_h.push_back(q);
        src_h.push_back(qs);
        pt_h.push_back(j);
      }
    }
    mw = static_cast<int64_t>(map_h.size());
    nq = static_cast<int64_t>(qlist_h.size());
    if (mw == 0) return;
    if (mw > (1LL << 31) - 1) throw CudaError("IV working set above 2^31 points");
    ntiles = static_cast<int32_t>((mw + kTile - 1) / kTile);
    tiles_h.assign(static_cast<size_t>(ntiles), TileDev{});
    const OptDev* ho = src->h_opts.as<OptDev>();
    int64_t off = 0, xoff = 0, foff = 0;
    for (int32_t t = 0; t < ntiles; ++t) {
      TileDev& td = tiles_h[t];
      td.first = t * kTile;
      td.count = static_cast<int32_t>(std::min<int64_t>(kTile, mw - td.first));
      int32_t nx = 0, nt = 0;
      for (int l = 0; l < td.count; ++l) {
        const OptDev& o = ho[src_h[td.first + l]];
        nx = std::max(nx, o.n);
        nt = std::max(nt, o.nt);
      }
      td.nx = nx;
      td.nt = nt;
      td.off = off;
      td.xoff = xoff;
      td.foff = foff;
      off += static_cast<int64_t>(A_COUNT) * nx * kTile;
      xoff += static_cast<int64_t>(nx) * kTile;
      foff += static_cast<int64_t>(nx) * kTile;
    }
    pool_doubles = off;
    check(cudaMemcpyAsync(d_tiles.get(sizeof(TileDev) * ntiles), tiles_h.data(),
                          sizeof(TileDev) * ntiles, cudaMemcpyHostToDevice, st),
          "H2D working tiles");
    check(cudaMemcpyAsync(d_map.get(sizeof(int32_t) * mw), map_h.data(), sizeof(int32_t) * mw,
                          cudaMemcpyHostToDevice, st),
          "H2D working map");
    if (smap)
      check(cudaMemcpyAsync(d_src.get(sizeof(int32_t) * mw), src_h.data(), sizeof(int32_t) * mw,
                            cudaMemcpyHostToDevice, st),
            "H2D working source map");
    check(cudaMemcpyAsync(d_pt.get(sizeof(int32_t) * mw), pt_h.data(), sizeof(int32_t) * mw,
                          cudaMemcpyHostToDevice, st),
          "H2D working points");
    check(cudaMemcpyAsync(d_qlist.get(sizeof(int32_t) * nq), qlist_h.data(), sizeof(int32_t) * nq,
                          cudaMemcpyHostToDevice, st),
          "H2D quote list");
    check(cudaMemcpyAsync(d_qbase.get(sizeof(int32_t) * nq), qbase_h.data(), sizeof(int32_t) * nq,
                          cudaMemcpyHostToDevice, st),
          "H2D quote slots");
    d_opts.get(sizeof(OptDev) * mw);
    d_xs.get(sizeof(double) * xoff);
    d_sigma.get(sizeof(double) * mw);
    d_active.get(sizeof(int32_t) * mw);
    d_pool.get(sizeof(double) * off);
    d_flags.get(static_cast<size_t>(foff));
    d_mode.get(sizeof(int32_t) * mw);
    d_status.get(sizeof(int32_t) * mw);
    d_out4.get(sizeof(double) * 4 * mw);
    if (tangent) d_tpool.get(sizeof(double) * static_cast<size_t>(tan_pool_doubles(1, off)));
    iv_gather_kernel<<<static_cast<int>((mw + 255) / 256), 256, 0, st>>>(
        static_cast<int>(mw), d_map.as<int32_t>(), smap ? d_src.as<int32_t>() : nullptr,
        d_pt.as<int32_t>(), src->d_tiles.as<TileDev>(), src->d_opts.as<OptDev>(),
        src->d_xs.as<double>(), d_tiles.as<TileDev>(), d_opts.as<OptDev>(), d_xs.as<double>(),
        next_sig, d_sigma.as<double>(), d_active.as<int32_t>());
    check(cudaGetLastError(), "iv_gather launch");
    tv_first = 0x7fffffff;
    if (smap) return;  // the coarse batch holds no time-varying quote
    for (int64_t k = 0; k < mw; ++k)
      if (map_h[k] >= b->mc.tv_first) {
        tv_first = static_cast<int32_t>(k);
        break;
      }
    if (tv_first < mw) {
      const int64_t ntv = mw - tv_first;
      iv_gather_tv_kernel<<<static_cast<int>((ntv + 255) / 256), 256, 0, st>>>(
          static_cast<int>(ntv), d_map.as<int32_t>() + tv_first, b->mc.tv_first,
          b->d_tv.as<TvDev>(), static_cast<TvDev*>(d_tv.get(sizeof(TvDev) * ntv)));
      check(cudaGetLastError(), "iv_gather_tv launch");
    }
  }
};

MangoStatus solve_iv(MangoGpuContext* ctx, const MangoIvQuery* queries, uint64_t n,
                     const MangoGpuGrid* grids, uint64_t grid_stride, const MangoIvConfig* config,
                     int32_t method, MangoIvBatchSlot* out, uint64_t* out_failed, MangoError* err) {
  if (!ctx || (n > 0 && (!queries || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, queries or out");
    return MANGO_ERR_VALIDATION;
  }
  if (!grids) {
    set_err(err, MANGO_ERR_VALIDATION,
            "IV needs a fixed grid per quote (MANGO_GPU_GRID_FIXED_N_AT_VOL, _SINH or _UNIFORM)");
    return MANGO_ERR_VALIDATION;
  }
  if (method != MANGO_GPU_IV_BRENT && method != MANGO_GPU_IV_SECANT &&
      method != MANGO_GPU_IV_NEWTON) {
    set_err(err, MANGO_ERR_VALIDATION, "unknown IV method");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 30)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^30 quotes");
    return MANGO_ERR_VALIDATION;
  }
  const double tol = (config && config->brent_tol_abs > 0.0) ? config->brent_tol_abs : 1e-6;
  const int max_iter = (config && config->max_iter > 0) ? config->max_iter : 100;
  const char* trace_env = std::getenv("MANGO_GPU_IV_TRACE");
  const bool trace = trace_env && trace_env[0] == '1';
  MangoGpuBatch* b = nullptr;
  MangoGpuBatch* bc = nullptr;  // Newton: the coarse grids
  const auto t_start = Clock::now();
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int64_t nn = static_cast<int64_t>(n);
    // Quotes -> pricing parameters (volatility is the unknown; the grid is
    // fixed per quote and must not depend on it).
    std::vector<MangoPricingParams> pp(static_cast<size_t>(nn));
    std::vector<int32_t> vstatus(static_cast<size_t>(nn), MANGO_OK);
    std::vector<std::string> vmsg(static_cast<size_t>(nn));
    std::vector<double> upper(static_cast<size_t>(nn), 1.5);
    for (int64_t i = 0; i < nn; ++i) {
      const MangoIvQuery& q = queries[i];
      const MangoGpuGrid& g = grids[grid_stride ? i : 0];
      MangoPricingParams& p = pp[i];
      std::memset(&p, 0, sizeof(p));
      p.spot = q.spot;
      p.strike = q.strike;
      p.maturity = q.maturity;
      p.dividend_yield = q.dividend_yield;
      p.rate_const = q.rate_const;
      p.tenor_points = q.tenor_points;
      p.n_tenor_points = q.n_tenor_points;
      p.dividends = q.dividends;
      p.n_dividends = q.n_dividends;
      p.option_type = q.option_type;
      p.volatility = 0.2;  // placeholder; every evaluation overrides it
      vstatus[i] = iv_query_status(q, &vmsg[i]);
      if (vstatus[i] == MANGO_OK && g.kind != MANGO_GPU_GRID_FIXED_N_AT_VOL &&
          g.kind != MANGO_GPU_GRID_SINH && g.kind != MANGO_GPU_GRID_UNIFORM) {
        vstatus[i] = MANGO_ERR_VALIDATION;
        vmsg[i] = "IV needs a volatility-independent grid (FIXED_N_AT_VOL, SINH or UNIFORM)";
      }
      if (vstatus[i] != MANGO_OK) p.spot = -1.0;  // keeps the quote out of the device batch
      // IVSolver::solve_brent upper bracket by time-value ratio (iv_solver.cpp:137-148)
      const bool put = q.option_type == MANGO_PUT;
      const double intrinsic =
          put ? std::max(q.strike - q.spot, 0.0) : std::max(q.spot - q.strike, 0.0);
      const double ratio = (q.market_price - intrinsic) / q.market_price;
      upper[i] = ratio > 0.5 ? 3.0 : (ratio > 0.2 ? 2.0 : 1.5);
    }
    // The batches live in the context between solves.  Their own march
    // buffers are never allocated: every evaluation runs on a packed
    // working set.
    for (MangoGpuBatch*& ib : ctx->iv_batch)
      if (!ib) {
        ib = new MangoGpuBatch();
        ib->march_buffers = false;
      }
    // Newton's coarse grids only steer the iteration (every root is
    // settled on the quote's own grid), so they are generated on the
    // device.  The own grids (host sinh, bit for bit the reference's) are
    // first needed after the coarse rounds: Newton fills them on a host
    // thread while those run.
    ctx->iv_batch[1]->device_grids = true;
    ctx->iv_batch[0]->defer_grids = method == MANGO_GPU_IV_NEWTON;
    b = create_batch(ctx, pp.data(), nn, grids, grid_stride, nullptr, ctx->iv_batch[0]);
    double host_prep_ms = b->host_prep_ms;
    const int64_t m = static_cast<int64_t>(b->order.size());
    // Newton: the same quotes on coarse grids of the same kind (2/5 of the
    // space points, an eighth of the steps; an estimated step count stays
    // estimated), and the map from b's sorted order to bc's.
    std::vector<int32_t> cmap;
    if (method == MANGO_GPU_IV_NEWTON && m > 0) {
      std::vector<MangoPricingParams> pc(pp);
      std::vector<MangoGpuGrid> gc(static_cast<size_t>(nn));
      for (int64_t i = 0; i < nn; ++i) {
        MangoGpuGrid g = grids[grid_stride ? i : 0];
        g.n_space = std::max<int64_t>(21, (2 * g.n_space / 5) | 1);
        if (g.n_time > 0) g.n_time = std::max<int64_t>(16, g.n_time / 8);
        gc[i] = g;
        if (vstatus[i] != MANGO_OK || time_varying(pp[i])) pc[i].spot = -1.0;
      }
      bc = create_batch(ctx, pc.data(), nn, gc.data(), 1, nullptr, ctx->iv_batch[1]);
      host_prep_ms += bc->host_prep_ms;
      std::vector<int32_t> pos(static_cast<size_t>(nn), -1);
      for (size_t s2 = 0; s2 < bc->order.size(); ++s2) pos[bc->order[s2]] = static_cast<int32_t>(s2);
      cmap.assign(static_cast<size_t>(m), -1);
      for (int64_t s2 = 0; s2 < m; ++s2) cmap[s2] = pos[b->order[s2]];
    }
    // Deferred own grids: the options' upload must have left the pinned
    // buffer before the worker writes their boundary data into it.
    std::thread grid_worker;
    std::exception_ptr grid_err;
    struct JoinGuard {
      std::thread& t;
      ~JoinGuard() {
        if (t.joinable()) t.join();
      }
    } grid_guard{grid_worker};
    bool grids_pending = b->grids_pending;
    if (grids_pending) {
      check(cudaStreamSynchronize(ctx->stream), "stream synchronize");
      grid_worker = std::thread([b, &grid_err] {
        try {
          fill_batch_grids(b);
        } catch (...) {
          grid_err = std::current_exception();
        }
      });
    }
    auto grids_ready = [&] {
      if (!grids_pending) return;
      const auto tw = Clock::now();
      grid_worker.join();
      if (grid_err) std::rethrow_exception(grid_err);
      upload_batch_grids(b);
      grids_pending = false;
      host_prep_ms += ms_since(tw);
    };
    std::vector<IvOut> hr(static_cast<size_t>(m));
    int64_t launches = 0, evaluations = 0;
    int64_t level_evals[kLevels] = {0, 0};
    double slot_evals = 0, eval_ms = 0, pack_ms = 0;
    if (m > 0) {
      cudaStream_t st = ctx->stream;
      std::vector<double> hi_sorted(static_cast<size_t>(m)), px(static_cast<size_t>(m)),
          mat(static_cast<size_t>(m));
      for (int64_t s = 0; s < m; ++s) {
        const MangoIvQuery& q = queries[b->order[s]];
        hi_sorted[s] = upper[b->order[s]];
        px[s] = q.market_price;
        mat[s] = q.maturity;
      }
      DevBuf &d_state = ctx->iv_dev[0], &d_res = ctx->iv_dev[1], &d_next = ctx->iv_dev[2],
             &d_npts = ctx->iv_dev[3], &d_hi = ctx->iv_dev[4], &d_px = ctx->iv_dev[5],
             &d_mat = ctx->iv_dev[6], &d_lev = ctx->iv_dev[7];
      HostBuf &h_npts = ctx->iv_host[0], &h_lev = ctx->iv_host[1], &h_sig1 = ctx->iv_host[2];
      IvDev* S = static_cast<IvDev*>(d_state.get(sizeof(IvDev) * m));
      IvOut* R = static_cast<IvOut*>(d_res.get(sizeof(IvOut) * m));
      double* next_sig = static_cast<double*>(d_next.get(sizeof(double) * kMaxPts * m));
      int32_t* npts = static_cast<int32_t*>(d_npts.get(sizeof(int32_t) * m));
      int32_t* hnpts = static_cast<int32_t*>(h_npts.get(sizeof(int32_t) * m));
      int32_t* lev = static_cast<int32_t*>(d_lev.get(sizeof(int32_t) * m));
      int32_t* hlev = static_cast<int32_t*>(h_lev.get(sizeof(int32_t) * m));
      double* hsig1 = static_cast<double*>(h_sig1.get(sizeof(double) * m));
      double* dhi = static_cast<double*>(d_hi.get(sizeof(double) * m));
      double* dpx = static_cast<double*>(d_px.get(sizeof(double) * m));
      double* dmat = static_cast<double*>(d_mat.get(sizeof(double) * m));
      check(cudaMemcpyAsync(dhi, hi_sorted.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dpx, px.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dmat, mat.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
      const int tb = 256;
      auto grid_of = [&](int64_t c) { return static_cast<int>((c + tb - 1) / tb); };
      // Points per quote: one wave of lanes (every resident march warp, one
      // tile each) spread over the quotes left, 1 .. kMaxPts.  Once the
      // working set no longer fits L2 a single round costs about as much
      // with one warp per SM sub-partition as with all of them resident, so
      // the full wave converges the tail in fewer evaluations (measured:
      // 262,144 quotes in 11 evaluations instead of 13, 128 k against
      // 117 k IV/s, identical statuses).
      const int64_t wave =
          static_cast<int64_t>(ctx->num_sms) * ctx->march_blocks_per_sm * 4 * kTile;
      auto points_for = [&](int64_t quotes) {
        if (method == MANGO_GPU_IV_BRENT) return 1;
        return static_cast<int>(
            std::max<int64_t>(1, std::min<int64_t>(kMaxPts, wave / std::max<int64_t>(quotes, 1))));
      };
      iv_init_kernel<<<grid_of(m), tb, 0, st>>>(
          static_cast<int>(m), method, points_for(m),
          static_cast<int>(std::min<int64_t>(b->mc.tv_first, m)), b->d_opts.as<OptDev>(), dmat,
          dpx, dhi, S, R, next_sig, npts, lev);
      check(cudaGetLastError(), "iv_init launch");
      ++launches;
      cudaEvent_t ev[2] = {nullptr, nullptr};
      struct Events {
        cudaEvent_t* e;
        ~Events() {
          for (int j = 0; j < 2; ++j)
            if (e[j]) cudaEventDestroy(e[j]);
        }
      } events{ev};
      for (cudaEvent_t& e : ev) check(cudaEventCreate(&e), "cudaEventCreate");
      // Working sets by level: coarse grids with the volatility tangent
      // (Newton's first evaluations), the own grids without it.
      WorkSet ws[kLevels];
      for (int L = 0; L < kLevels; ++L) {
        ws[L].borrow(ctx->iv_ws[L]);
        ws[L].b = b;
        ws[L].src = (L == kLevelCoarse) ? bc : b;
        ws[L].smap = (L == kLevelCoarse) ? &cmap : nullptr;
        ws[L].tangent = L == kLevelCoarse;
        ws[L].st = st;
      }
      std::vector<int32_t> active(static_cast<size_t>(m));
      std::iota(active.begin(), active.end(), 0);
      std::vector<int32_t> lists[kLevels];
      double level_slot_evals[kLevels] = {0.0, 0.0};
      // Fast or Newton evaluations, then Brent's two bracket ends and max_iter steps.
      const int max_evals =
          (method == MANGO_GPU_IV_BRENT ? 0 : kFastMaxBracketEvals + kCoarseEvals) + max_iter + 3;
      for (int e = 0; e < max_evals; ++e) {
        check(cudaMemcpyAsync(hnpts, npts, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st),
              "D2H points");
        check(cudaMemcpyAsync(hlev, lev, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st),
              "D2H levels");
        // Few quotes left (the tail): their first trial points too, to order
        // the working set below.
        const bool tail = static_cast<int64_t>(active.size()) <= kTailQuotes;
        if (tail)
          check(cudaMemcpy2DAsync(hsig1, sizeof(double), next_sig, sizeof(double) * kMaxPts,
                                  sizeof(double), static_cast<size_t>(m), cudaMemcpyDeviceToHost, st),
                "D2H trial points");
        check(cudaStreamSynchronize(st), "stream synchronize");
        const auto tp = Clock::now();
        for (auto& l : lists) l.clear();
        std::vector<int32_t> still;
        still.reserve(active.size());
        for (int32_t q : active)
          if (hnpts[q] > 0) {
            still.push_back(q);
            lists[std::min(std::max(hlev[q], 0), kLevels - 1)].push_back(q);
          }
        active.swap(still);
        if (tail) {
          // The tail's quotes are a sparse, scattered subset whose trial
          // volatilities differ from the ones the batch was sorted by: order
          // them again by type and ln(S/K) / (sigma sqrt(T)) at their next
          // trial point, so that the lanes of a tile meet the obstacle at
          // similar rows (as the pricing batch's sort arranges).
          // (keys computed once per quote, not per comparison)
          const OptDev* ho = b->h_opts.as<OptDev>();
          struct TailKey {
            int32_t put;
            double k;
            int32_t q;
          };
          std::vector<TailKey> keys;
          for (auto& l : lists) {
            keys.resize(l.size());
            for (size_t j = 0; j < l.size(); ++j) {
              const int32_t q = l[j];
              const double sg = hsig1[q] > 0.0 ? hsig1[q] : 0.2;
              keys[j] = TailKey{ho[q].is_put,
                                std::log(ho[q].spot / ho[q].strike) / (sg * std::sqrt(mat[q])), q};
            }
            std::sort(keys.begin(), keys.end(), [](const TailKey& a, const TailKey& c) {
              if (a.put != c.put) return a.put < c.put;
              return a.k != c.k ? a.k < c.k : a.q < c.q;
            });
            for (size_t j = 0; j < l.size(); ++j) l[j] = keys[j].q;
          }
        }
        if (!lists[kLevelPlain].empty()) grids_ready();
        int64_t nq_all = 0;
        for (int L = 0; L < kLevels; ++L) {
          ws[L].pack(lists[L], hnpts, next_sig);
          nq_all += ws[L].nq;
        }
        pack_ms += ms_since(tp);
        if (nq_all == 0) break;
        const int k_next = points_for(nq_all);
        check(cudaMemsetAsync(b->d_queue.p, 0, sizeof(int) * 4, st), "memset queue");
        check(cudaEventRecord(ev[0], st), "event");
        for (int L = 0; L < kLevels; ++L) {
          WorkSet& w = ws[L];
          if (w.mw == 0) continue;
          MarchConst mc = w.src->mc;
          mc.value_only = 1;
          mc.sigma = w.d_sigma.as<double>();
          mc.active = w.d_active.as<int32_t>();
          mc.tv_first = w.tv_first;
          const int ntiles = w.ntiles, threads = ntiles * kTile;
          const TileDev* tiles = w.d_tiles.as<TileDev>();
          const OptDev* wopts = w.d_opts.as<OptDev>();
          const double* xs = w.d_xs.as<double>();
          int* queue = b->d_queue.as<int>() + L;
          if (w.tangent) {
            TanConst tc{};
            tc.dirs[0] = kDirSigma;
            tan_launch(1, st, ctx->num_sms, tiles, ntiles, wopts, xs, w.d_pool.as<double>(),
                       w.d_tpool.as<double>(), w.d_flags.as<uint8_t>(), w.d_mode.as<int32_t>(),
                       w.d_status.as<int32_t>(), queue, tc, mc, w.d_out4.as<double>());
            launches += 5;  // gather, prep, tangent prep, march, outputs
          } else {
            const int blocks = std::max(
                1, std::min<int>(ctx->num_sms * ctx->march_blocks_per_sm, (ntiles + 3) / 4));
            // few points left: one warp per option (wmarch.cu).  A tail
            // round's thread march was measured at about twice the time of a
            // pricing batch of its size (trial volatilities far from the
            // grid's slow some lanes, and a tile waits for its slowest), so
            // its estimate counts double (MANGO_GPU_IV_TAIL_SCALE: that
            // factor, for sweeps).
            double tail_scale = 2.0;
            if (const char* e = std::getenv("MANGO_GPU_IV_TAIL_SCALE"))
              if (std::atof(e) > 0.0) tail_scale = std::atof(e);
            const WarpPlan plan = plan_warp_tiles(
                w.tiles_h.data(), ntiles, w.tv_first < w.mw ? w.tv_first / kTile : ntiles,
                ctx->num_sms,
                static_cast<int64_t>(active.size()) <= kTailQuotes ? tail_scale : 1.0);
            const int nwt = static_cast<int>(plan.tiles.size());
            if (nwt > 0) {
              check(cudaMemcpyAsync(w.d_wt.get(sizeof(int32_t) * nwt), plan.tiles.data(),
                                    sizeof(int32_t) * nwt, cudaMemcpyHostToDevice, st),
                    "H2D warp tiles");
              check(cudaMemcpyAsync(w.d_twarp.get(static_cast<size_t>(ntiles)), plan.flag.data(),
                                    static_cast<size_t>(ntiles), cudaMemcpyHostToDevice, st),
                    "H2D warp flags");
              mc.tile_warp = w.d_twarp.as<uint8_t>();
            }
            prep_kernel<<<(threads + 127) / 128, 128, 0, st>>>(tiles, ntiles, wopts, xs,
                                                               w.d_pool.as<double>(),
                                                               w.d_flags.as<uint8_t>(),
                                                               w.d_mode.as<int32_t>(), mc);
            if (nwt < ntiles) {
              // tile hand-off (march.cuh), as in the pricing batch's launch
              MarchConst mh = mc;
              const char* he = std::getenv("MANGO_GPU_HANDOFF");
              if (!(he && he[0] == '0')) {
                const int cap = 4 * ntiles + 1024;
                const size_t bytes = 16 + sizeof(unsigned long long) * static_cast<size_t>(cap) +
                                     static_cast<size_t>(ntiles);
                char* h = static_cast<char*>(w.d_ho.get(bytes));
                check(cudaMemsetAsync(h, 0, bytes, st), "memset hand-off");
                mh.ho_ctl = reinterpret_cast<int*>(h);
                mh.ho_slot = reinterpret_cast<unsigned long long*>(h + 16);
                mh.ho_moved = reinterpret_cast<uint8_t*>(h + 16 + sizeof(unsigned long long) * cap);
                mh.ho_cap = cap;
                mh.ho_total = ntiles;
              }
              march_kernel<<<blocks, 128, 0, st>>>(tiles, ntiles, wopts, w.d_pool.as<double>(),
                                                   w.d_flags.as<uint8_t>(), w.d_mode.as<int32_t>(),
                                                   w.d_status.as<int32_t>(), queue, mh);
            }
            wmarch_launch(st, ctx->num_sms, tiles, w.d_wt.as<int32_t>(), nwt, wopts,
                          w.d_pool.as<double>(), w.d_flags.as<uint8_t>(), w.d_mode.as<int32_t>(),
                          w.d_status.as<int32_t>(), b->d_queue.as<int>() + 3, mc, plan.R);
            if (w.tv_first < w.mw) {
              const int t0 = w.tv_first / kTile;
              const int tvb = std::max(1, std::min<int>(ctx->num_sms * 8, (ntiles - t0 + 3) / 4));
              march_tv_kernel<<<tvb, 128, 0, st>>>(
                  tiles, t0, ntiles, wopts, w.d_tv.as<TvDev>(), b->d_tv_tp.as<double>(),
                  b->d_tv_curve.as<double>(), b->d_tv_ev.as<double>(), xs, w.d_pool.as<double>(),
                  w.d_mode.as<int32_t>(), w.d_status.as<int32_t>(), mc);
              ++launches;
            }
            outputs_kernel<<<(threads + 127) / 128, 128, 0, st>>>(
                tiles, ntiles, wopts, xs, w.d_pool.as<double>(), w.d_mode.as<int32_t>(),
                w.d_status.as<int32_t>(), mc, w.d_out4.as<double>());
            launches += 4;  // gather, prep, march, outputs
          }
          iv_step_kernel<<<grid_of(w.nq), tb, 0, st>>>(
              static_cast<int>(w.nq), w.d_qlist.as<int32_t>(), w.d_qbase.as<int32_t>(), k_next, S,
              R, b->d_opts.as<OptDev>(), dmat, dhi, w.d_out4.as<double>(),
              w.d_status.as<int32_t>(), w.d_sigma.as<double>(), dpx, next_sig, npts, tol,
              max_iter, trace ? 1 : 0, w.tangent ? 1 : 0, lev);
          check(cudaGetLastError(), "iv evaluation launch");
          launches += 1;
          level_slot_evals[L] += static_cast<double>(w.mw);
          slot_evals += static_cast<double>(w.mw);
        }
        check(cudaEventRecord(ev[1], st), "event");
        check(cudaStreamSynchronize(st), "stream synchronize");
        float ms = 0.f;
        check(cudaEventElapsedTime(&ms, ev[0], ev[1]), "event time");
        eval_ms += ms;
        evaluations += 1;
        if (trace)
          std::fprintf(stderr,
                       "iv evaluation %d: quotes coarse %lld / own %lld, points %lld / %lld, "
                       "next %d per quote, %.3f ms\n",
                       e, static_cast<long long>(ws[kLevelCoarse].nq),
                       static_cast<long long>(ws[kLevelPlain].nq),
                       static_cast<long long>(ws[kLevelCoarse].mw),
                       static_cast<long long>(ws[kLevelPlain].mw), k_next, ms);
      }
      for (int L = 0; L < kLevels; ++L) level_evals[L] = static_cast<int64_t>(level_slot_evals[L]);
      check(cudaMemcpyAsync(hr.data(), R, sizeof(IvOut) * m, cudaMemcpyDeviceToHost, st), "D2H results");
      check(cudaStreamSynchronize(st), "stream synchronize");
    }
    uint64_t failed = 0;
    std::string first;
    for (int64_t i = 0; i < nn; ++i) {
      MangoIvBatchSlot& o = out[i];
      std::memset(&o, 0, sizeof(o));
      o.status = vstatus[i];
      if (vstatus[i] != MANGO_OK && first.empty()) first = vmsg[i];
    }
    for (int64_t s = 0; s < m; ++s) {
      MangoIvBatchSlot& o = out[b->order[s]];
      const IvOut& r = hr[s];
      switch (r.code) {
        case kIvOk: o.status = MANGO_OK; break;
        case kIvBracket: o.status = MANGO_ERR_BRACKETING; break;
        case kIvMaxIter: o.status = MANGO_ERR_NO_CONVERGENCE; break;
        default: o.status = MANGO_ERR_SOLVER; break;
      }
      o.success.implied_vol = r.code == kIvOk ? r.root : NAN;
      o.success.iterations = static_cast<uint64_t>(r.iter);
      o.success.final_error = r.ferr;
      o.success.has_vega = r.code == kIvOk && std::isfinite(r.vega) ? 1 : 0;
      o.success.vega = o.success.has_vega ? r.vega : 0.0;
      o.success.used_rate_approximation = 0;
    }
    for (int64_t i = 0; i < nn; ++i) failed += out[i].status != MANGO_OK;
    ctx->stats = Stats{};
    ctx->stats.host_prep_ms = host_prep_ms;
    ctx->stats.prep_ms = pack_ms;
    ctx->stats.march_ms = eval_ms;
    ctx->stats.total_ms = ms_since(t_start);
    ctx->stats.kernel_launches = launches;
    ctx->stats.options = static_cast<int64_t>(slot_evals);
    for (int L = 0; L < kLevels; ++L) ctx->stats.iv_evals[L] = level_evals[L];
    ctx->stats.tiles = evaluations;
    ctx->stats.algo_flops = m > 0 ? b->algo_flops * slot_evals / static_cast<double>(m) : 0.0;
    if (out_failed) *out_failed = failed;
    if (failed && err) set_err(err, MANGO_OK, first.empty() ? "root finding failed" : first);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

}  // namespace
}  // namespace mgpu

extern "C" MangoStatus mango_gpu_solve_iv_batch(MangoGpuContext* ctx, const MangoIvQuery* queries,
                                                uint64_t n, const MangoGpuGrid* grids,
                                                uint64_t grid_stride, const MangoIvConfig* config,
                                                MangoIvBatchSlot* out, uint64_t* out_failed,
                                                MangoError* err) {
  return mgpu::solve_iv(ctx, queries, n, grids, grid_stride, config, MANGO_GPU_IV_BRENT, out,
                        out_failed, err);
}

extern "C" MangoStatus mango_gpu_solve_iv_batch_method(MangoGpuContext* ctx,
                                                       const MangoIvQuery* queries, uint64_t n,
                                                       const MangoGpuGrid* grids,
                                                       uint64_t grid_stride,
                                                       const MangoIvConfig* config, int32_t method,
                                                       MangoIvBatchSlot* out, uint64_t* out_failed,
                                                       MangoError* err) {
  return mgpu::solve_iv(ctx, queries, n, grids, grid_stride, config, method, out, out_failed, err);
}
