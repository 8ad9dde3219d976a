// grid_host.cpp -- see grid_host.hpp.  Reference formulas, reference order.
#include "grid_host.hpp"

#include <algorithm>

#include <cfloat>
#include <cmath>
#include <vector>

namespace mgpu {

namespace {

// sinh(c (i / (n - 1) - 0.5)) / sinh(c / 2) for i in [0, n): the same for
// every grid with this concentration and point count, so a batch of grids
// that differ only in their bounds evaluates it once per host thread.  The
// values are computed by the same expression, in the same order, as an
// uncached evaluation: the grids stay bit for bit the same.
const double* sinh_profile(double c, int64_t n) {
  thread_local double cached_c = 0.0;
  thread_local int64_t cached_n = -1;
  thread_local std::vector<double> st;
  if (cached_n != n || !(cached_c == c) || std::signbit(cached_c) != std::signbit(c)) {
    const double nm1 = static_cast<double>(n - 1);
    const double shc = std::sinh(c / 2.0);
    st.resize(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) {
      const double eta = static_cast<double>(i) / nm1;
      st[static_cast<size_t>(i)] = std::sinh(c * (eta - 0.5)) / shc;
    }
    cached_c = c;
    cached_n = n;
  }
  return st.data();
}

}  // namespace

Accuracy default_accuracy() {
  Accuracy a;
  a.alpha = 2.0 * std::asinh(5.0 / std::sqrt(2.0));  // grid_spec_types.hpp:15-19
  return a;
}

namespace {

// Pairwise cluster merge until stable (grid.hpp:191-234).
void merge_clusters(GridSpec* s) {
  bool merged = true;
  while (merged) {
    merged = false;
    for (int i = 0; i < s->n_clusters && !merged; ++i) {
      for (int j = i + 1; j < s->n_clusters && !merged; ++j) {
        const double dx = std::fabs(s->c_center[i] - s->c_center[j]);
        const double a_avg = (s->c_alpha[i] + s->c_alpha[j]) / 2.0;
        const double thr = 0.3 / a_avg;
        if (dx <= thr + 100.0 * DBL_EPSILON) {
          const double tw = s->c_weight[i] + s->c_weight[j];
          const double wi = s->c_weight[i] / tw;
          const double wj = s->c_weight[j] / tw;
          const double center = wi * s->c_center[i] + wj * s->c_center[j];
          const double alpha = wi * s->c_alpha[i] + wj * s->c_alpha[j];
          s->c_center[i] = center;
          s->c_alpha[i] = alpha;
          s->c_weight[i] = tw;
          for (int k = j; k + 1 < s->n_clusters; ++k) {
            s->c_center[k] = s->c_center[k + 1];
            s->c_alpha[k] = s->c_alpha[k + 1];
            s->c_weight[k] = s->c_weight[k + 1];
          }
          --s->n_clusters;
          merged = true;
        }
      }
    }
  }
}

// Endpoint clamp plus forward/backward minimum-spacing passes (grid.hpp:240-262).
void monotone(double* p, int64_t n, double lo, double hi) {
  if (n < 2) return;
  const double ms = (hi - lo) / static_cast<double>(n * 100);
  p[0] = lo;
  p[n - 1] = hi;
  for (int64_t i = 1; i < n - 1; ++i)
    if (p[i] <= p[i - 1] + ms) p[i] = p[i - 1] + ms;
  for (int64_t i = n - 2; i > 0; --i)
    if (p[i] >= p[i + 1] - ms) p[i] = p[i + 1] - ms;
}

}  // namespace

GridSpec sinh_spec(double x_min, double x_max, int64_t n, double alpha) {
  GridSpec s;
  s.type = GridSpec::Sinh;
  s.x_min = x_min;
  s.x_max = x_max;
  s.n = n;
  s.concentration = alpha;
  return s;
}

GridSpec uniform_spec(double x_min, double x_max, int64_t n) {
  GridSpec s;
  s.type = GridSpec::Uniform;
  s.x_min = x_min;
  s.x_max = x_max;
  s.n = n;
  return s;
}

void generate_grid(const GridSpec& s, double* x) {
  const int64_t n = s.n;
  const double lo = s.x_min, hi = s.x_max;
  const double nm1 = static_cast<double>(n - 1);
  switch (s.type) {
    case GridSpec::Uniform: {
      const double dx = (hi - lo) / nm1;
      for (int64_t i = 0; i < n; ++i) x[i] = lo + static_cast<double>(i) * dx;
      return;
    }
    case GridSpec::Log: {
      const double l0 = std::log(lo), l1 = std::log(hi);
      const double dl = (l1 - l0) / nm1;
      for (int64_t i = 0; i < n; ++i) x[i] = std::exp(l0 + static_cast<double>(i) * dl);
      return;
    }
    case GridSpec::Sinh: {
      const double* st = sinh_profile(s.concentration, n);
      for (int64_t i = 0; i < n; ++i) x[i] = lo + (hi - lo) * ((1.0 + st[i]) / 2.0);
      return;
    }
    case GridSpec::MultiSinh: {
      const double range = hi - lo;
      if (s.n_clusters == 1) {
        const double c = s.c_alpha[0], center = s.c_center[0];
        const double shc = std::sinh(c / 2.0);
        const double eta_c = (center - lo) / range;
        if (std::fabs(eta_c - 0.5) < 1e-10) {
          const double* st = sinh_profile(c, n);
          for (int64_t i = 0; i < n; ++i) x[i] = lo + range * ((1.0 + st[i]) / 2.0);
        } else {
          const double off = center - (lo + hi) / 2.0;
          for (int64_t i = 0; i < n; ++i) {
            const double eta = static_cast<double>(i) / nm1;
            const double st = std::sinh(c * (eta - eta_c)) / shc;
            x[i] = lo + range * ((1.0 + st) / 2.0) + off;
          }
          monotone(x, n, lo, hi);
        }
        return;
      }
      double total = 0.0;
      for (int k = 0; k < s.n_clusters; ++k) total += s.c_weight[k];
      // The per-cluster terms do not depend on the point: computed once
      // (same expressions, same values).
      double cw[4], cc[4], cshc[4], ceta[4], coff[4];
      for (int k = 0; k < s.n_clusters; ++k) {
        const double c = s.c_alpha[k], center = s.c_center[k];
        cw[k] = s.c_weight[k] / total;
        cc[k] = c;
        cshc[k] = std::sinh(c / 2.0);
        ceta[k] = (center - lo) / range;
        coff[k] = center - (lo + hi) / 2.0;
      }
      for (int64_t i = 0; i < n; ++i) {
        const double eta = static_cast<double>(i) / nm1;
        double acc = 0.0;
        for (int k = 0; k < s.n_clusters; ++k) {
          const double st = std::sinh(cc[k] * (eta - ceta[k])) / cshc[k];
          acc += cw[k] * (lo + range * ((1.0 + st) / 2.0) + coff[k]);
        }
        x[i] = acc;
      }
      monotone(x, n, lo, hi);
      return;
    }
  }
}

void estimate_spec(double spot, double strike, double maturity, double sigma,
                   const Accuracy& acc, GridSpec* spec) {
  // The spatial half of estimate_grid below (no trial grid, no step count).
  const double sst = sigma * std::sqrt(maturity);
  const double x0 = std::log(spot / strike);
  const double lo = x0 - acc.n_sigma * sst;
  const double hi = x0 + acc.n_sigma * sst;
  const double dx_target = sigma * std::sqrt(acc.tol);
  int64_t nx = static_cast<int64_t>(std::ceil((hi - lo) / dx_target));
  if (nx < acc.min_points) nx = acc.min_points;
  if (nx > acc.max_points) nx = acc.max_points;
  if (nx % 2 == 0) ++nx;
  GridSpec s;
  s.n = nx;
  s.x_min = lo;
  s.x_max = hi;
  s.n_clusters = 1;
  s.c_center[0] = x0;
  s.c_alpha[0] = acc.alpha;
  s.c_weight[0] = 0.5;
  if (0.0 >= lo && 0.0 <= hi) {
    s.c_center[1] = 0.0;
    s.c_alpha[1] = acc.alpha;
    s.c_weight[1] = 1.0;
    s.n_clusters = 2;
  }
  bool ok = nx >= 2 && lo < hi;
  for (int k = 0; k < s.n_clusters && ok; ++k)
    ok = s.c_alpha[k] > 0 && s.c_weight[k] > 0 && s.c_center[k] >= lo && s.c_center[k] <= hi;
  if (ok) {
    s.type = GridSpec::MultiSinh;
    merge_clusters(&s);
  } else {
    s = sinh_spec(lo, hi, nx, acc.alpha);
  }
  *spec = s;
}

void estimate_grid(double spot, double strike, double maturity, double sigma,
                   const Accuracy& acc, GridSpec* spec, int64_t* n_time,
                   std::vector<double>* scratch) {
  const double sst = sigma * std::sqrt(maturity);
  const double x0 = std::log(spot / strike);
  const double lo = x0 - acc.n_sigma * sst;
  const double hi = x0 + acc.n_sigma * sst;
  const double dx_target = sigma * std::sqrt(acc.tol);
  int64_t nx = static_cast<int64_t>(std::ceil((hi - lo) / dx_target));
  if (nx < acc.min_points) nx = acc.min_points;
  if (nx > acc.max_points) nx = acc.max_points;
  if (nx % 2 == 0) ++nx;

  GridSpec s;
  s.n = nx;
  s.x_min = lo;
  s.x_max = hi;
  s.n_clusters = 1;
  s.c_center[0] = x0;
  s.c_alpha[0] = acc.alpha;
  s.c_weight[0] = 0.5;
  if (0.0 >= lo && 0.0 <= hi) {
    s.c_center[1] = 0.0;
    s.c_alpha[1] = acc.alpha;
    s.c_weight[1] = 1.0;
    s.n_clusters = 2;
  }
  bool ok = nx >= 2 && lo < hi;
  for (int k = 0; k < s.n_clusters && ok; ++k)
    ok = s.c_alpha[k] > 0 && s.c_weight[k] > 0 && s.c_center[k] >= lo && s.c_center[k] <= hi;
  if (ok) {
    s.type = GridSpec::MultiSinh;
    merge_clusters(&s);
  } else {
    s = sinh_spec(lo, hi, nx, acc.alpha);
  }
  *spec = s;

  scratch->resize(static_cast<size_t>(nx));
  double* p = scratch->data();
  generate_grid(s, p);
  double dx_min = p[1] - p[0];
  for (int64_t i = 2; i < nx; ++i) {
    const double d = p[i] - p[i - 1];
    if (d < dx_min) dx_min = d;
  }
  const double dt = acc.c_t * dx_min;
  int64_t nt = static_cast<int64_t>(std::ceil(maturity / dt));
  if (nt > acc.max_steps) nt = acc.max_steps;
  *n_time = nt;
}

void time_points(double t0, double t1, double dt, std::vector<double> mandatory,
                 std::vector<double>* pts, int64_t* n_steps) {
  // TimeDomain::with_mandatory_points (src/pde/core/time_domain.hpp)
  std::vector<double> breaks;
  for (double t : mandatory)
    if (t > t0 + 1e-14 && t < t1 - 1e-14) breaks.push_back(t);
  std::sort(breaks.begin(), breaks.end());
  // std::unique: drop each point within 1e-14 of the last point kept
  size_t kept = 0;
  for (size_t i = 0; i < breaks.size(); ++i)
    if (kept == 0 || !(std::abs(breaks[kept - 1] - breaks[i]) < 1e-14)) breaks[kept++] = breaks[i];
  breaks.resize(kept);
  pts->clear();
  if (breaks.empty()) {
    *n_steps = static_cast<int64_t>(std::ceil((t1 - t0) / dt));
    return;
  }
  std::vector<double> bounds;
  bounds.push_back(t0);
  for (double b : breaks) bounds.push_back(b);
  bounds.push_back(t1);
  pts->push_back(t0);
  for (size_t seg = 0; seg + 1 < bounds.size(); ++seg) {
    const double s0 = bounds[seg], s1 = bounds[seg + 1];
    const double len = s1 - s0;
    int64_t n_sub = static_cast<int64_t>(std::ceil(len / dt));
    if (n_sub < 1) n_sub = 1;
    const double sub = len / static_cast<double>(n_sub);
    for (int64_t j = 1; j <= n_sub; ++j) pts->push_back(s0 + static_cast<double>(j) * sub);
  }
  *n_steps = static_cast<int64_t>(pts->size()) - 1;
}

void estimate_grid_div(double spot, double strike, double maturity, double sigma,
                       const Accuracy& acc, const std::vector<double>& taus, double max_dk,
                       GridSpec* spec, int64_t* n_time, std::vector<double>* tp,
                       std::vector<double>* scratch) {
  // estimate_pde_grid (src/option/grid_spec_types.cpp:37-118) with the
  // dividend widening of the lower bound and the mandatory time points.
  const double sst = sigma * std::sqrt(maturity);
  const double x0 = std::log(spot / strike);
  double lo = x0 - acc.n_sigma * sst;
  const double hi = x0 + acc.n_sigma * sst;
  const double dx_target = sigma * std::sqrt(acc.tol);
  int64_t nx = static_cast<int64_t>(std::ceil((hi - lo) / dx_target));
  if (nx < acc.min_points) nx = acc.min_points;
  if (nx > acc.max_points) nx = acc.max_points;
  if (nx % 2 == 0) ++nx;
  if (max_dk > 0.0 && std::exp(lo) > max_dk) {
    lo = std::log(std::exp(lo) - max_dk);
  } else if (max_dk > 0.0) {
    lo -= 1.0;
  }

  GridSpec s;
  s.n = nx;
  s.x_min = lo;
  s.x_max = hi;
  s.n_clusters = 1;
  s.c_center[0] = x0;
  s.c_alpha[0] = acc.alpha;
  s.c_weight[0] = 0.5;
  if (0.0 >= lo && 0.0 <= hi) {
    s.c_center[1] = 0.0;
    s.c_alpha[1] = acc.alpha;
    s.c_weight[1] = 1.0;
    s.n_clusters = 2;
  }
  bool ok = nx >= 2 && lo < hi;
  for (int k = 0; k < s.n_clusters && ok; ++k)
    ok = s.c_alpha[k] > 0 && s.c_weight[k] > 0 && s.c_center[k] >= lo && s.c_center[k] <= hi;
  if (ok) {
    s.type = GridSpec::MultiSinh;
    merge_clusters(&s);
  } else {
    s = sinh_spec(lo, hi, nx, acc.alpha);
  }
  *spec = s;

  scratch->resize(static_cast<size_t>(nx));
  double* p = scratch->data();
  generate_grid(s, p);
  double dx_min = p[1] - p[0];
  for (int64_t i = 2; i < nx; ++i) {
    const double d = p[i] - p[i - 1];
    if (d < dx_min) dx_min = d;
  }
  const double dt = acc.c_t * dx_min;
  int64_t nt = static_cast<int64_t>(std::ceil(maturity / dt));
  if (nt > acc.max_steps) nt = acc.max_steps;
  const double cap = maturity / static_cast<double>(acc.max_steps);
  const double dt_capped = (dt < cap) ? cap : dt;
  tp->clear();
  if (taus.empty()) {
    *n_time = nt;  // TimeDomain::from_n_steps
    return;
  }
  time_points(0.0, maturity, dt_capped, taus, tp, n_time);
}

void estimate_grid(double spot, double strike, double maturity, double sigma,
                   const Accuracy& acc, GridSpec* spec, int64_t* n_time, double* scratch,
                   int64_t cap) {
  // Identical to the vector overload above (estimate_pde_grid,
  // src/option/grid_spec_types.cpp:37-118) except for where the trial grid lives.
  const double sst = sigma * std::sqrt(maturity);
  const double x0 = std::log(spot / strike);
  const double lo = x0 - acc.n_sigma * sst;
  const double hi = x0 + acc.n_sigma * sst;
  const double dx_target = sigma * std::sqrt(acc.tol);
  int64_t nx = static_cast<int64_t>(std::ceil((hi - lo) / dx_target));
  if (nx < acc.min_points) nx = acc.min_points;
  if (nx > acc.max_points) nx = acc.max_points;
  if (nx % 2 == 0) ++nx;

  GridSpec s;
  s.n = nx;
  s.x_min = lo;
  s.x_max = hi;
  s.n_clusters = 1;
  s.c_center[0] = x0;
  s.c_alpha[0] = acc.alpha;
  s.c_weight[0] = 0.5;
  if (0.0 >= lo && 0.0 <= hi) {
    s.c_center[1] = 0.0;
    s.c_alpha[1] = acc.alpha;
    s.c_weight[1] = 1.0;
    s.n_clusters = 2;
  }
  bool ok = nx >= 2 && lo < hi;
  for (int k = 0; k < s.n_clusters && ok; ++k)
    ok = s.c_alpha[k] > 0 && s.c_weight[k] > 0 && s.c_center[k] >= lo && s.c_center[k] <= hi;
  if (ok) {
    s.type = GridSpec::MultiSinh;
    merge_clusters(&s);
  } else {
    s = sinh_spec(lo, hi, nx, acc.alpha);
  }
  *spec = s;
  *n_time = 0;
  if (nx > cap) return;
  generate_grid(s, scratch);
  double dx_min = scratch[1] - scratch[0];
  for (int64_t i = 2; i < nx; ++i) {
    const double d = scratch[i] - scratch[i - 1];
    if (d < dx_min) dx_min = d;
  }
  const double dt = acc.c_t * dx_min;
  int64_t nt = static_cast<int64_t>(std::ceil(maturity / dt));
  if (nt > acc.max_steps) nt = acc.max_steps;
  *n_time = nt;
}

}  // namespace mgpu
