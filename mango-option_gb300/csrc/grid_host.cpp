// grid_host.cpp -- see grid_host.hpp.  Reference formulas, reference order.
#include "grid_host.hpp"

#include <cfloat>
#include <cmath>

namespace mgpu {

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
      const double c = s.concentration;
      const double shc = std::sinh(c / 2.0);
      for (int64_t i = 0; i < n; ++i) {
        const double eta = static_cast<double>(i) / nm1;
        const double st = std::sinh(c * (eta - 0.5)) / shc;
        x[i] = lo + (hi - lo) * ((1.0 + st) / 2.0);
      }
      return;
    }
    case GridSpec::MultiSinh: {
      const double range = hi - lo;
      if (s.n_clusters == 1) {
        const double c = s.c_alpha[0], center = s.c_center[0];
        const double shc = std::sinh(c / 2.0);
        const double eta_c = (center - lo) / range;
        if (std::fabs(eta_c - 0.5) < 1e-10) {
          for (int64_t i = 0; i < n; ++i) {
            const double eta = static_cast<double>(i) / nm1;
            const double st = std::sinh(c * (eta - 0.5)) / shc;
            x[i] = lo + range * ((1.0 + st) / 2.0);
          }
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
      for (int64_t i = 0; i < n; ++i) {
        const double eta = static_cast<double>(i) / nm1;
        double acc = 0.0;
        for (int k = 0; k < s.n_clusters; ++k) {
          const double c = s.c_alpha[k], center = s.c_center[k];
          const double w = s.c_weight[k] / total;
          const double shc = std::sinh(c / 2.0);
          const double eta_c = (center - lo) / range;
          const double st = std::sinh(c * (eta - eta_c)) / shc;
          const double off = center - (lo + hi) / 2.0;
          acc += w * (lo + range * ((1.0 + st) / 2.0) + off);
        }
        x[i] = acc;
      }
      monotone(x, n, lo, hi);
      return;
    }
  }
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
