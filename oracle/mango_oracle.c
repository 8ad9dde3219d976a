/* mango_oracle.c -- CPU restatement of the reference's American-option hot
 * path.  TEST INFRASTRUCTURE ONLY (see mango_oracle.h): the checker for the
 * CUDA path, never part of it.  Compile with -ffp-contract=off so that the
 * only fused multiply-adds are the ones the reference spells as std::fma.
 *
 * Parity pinned against the reference itself: tests/golden/*.npz are written
 * by tests/golden/make_golden.py from the reference sources compiled by
 * oracle/ref/Makefile, and tests/test_oracle_pins.py compares this port with
 * them.
 */
#include "mango_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double dmax(double a, double b) { return (a < b) ? b : a; } /* std::max */
static double dmin(double a, double b) { return (b < a) ? b : a; } /* std::min */

/* ---------------------------------------------------------------- grids -- */

void mo_default_accuracy(mo_accuracy* acc) {
  /* GridAccuracyParams defaults, src/option/grid_spec_types.hpp:23-53;
   * optimal_sinh_alpha, grid_spec_types.hpp:15-19. */
  acc->n_sigma = 5.0;
  acc->alpha = 2.0 * asinh(5.0 / sqrt(2.0));
  acc->tol = 1e-2;
  acc->c_t = 0.75;
  acc->min_spatial_points = 100;
  acc->max_spatial_points = 1200;
  acc->max_time_steps = 5000;
}

/* GridSpec::merge_nearby_clusters, src/pde/core/grid.hpp:191-234. */
static void merge_clusters(mo_grid_spec* s) {
  int merged = 1;
  while (merged) {
    merged = 0;
    for (int i = 0; i < s->n_clusters && !merged; ++i) {
      for (int j = i + 1; j < s->n_clusters && !merged; ++j) {
        const double delta_x = fabs(s->c_center[i] - s->c_center[j]);
        const double alpha_avg = (s->c_alpha[i] + s->c_alpha[j]) / 2.0;
        const double threshold = 0.3 / alpha_avg;
        const double eps = 100.0 * DBL_EPSILON;
        if (delta_x <= threshold + eps) {
          const double tw = s->c_weight[i] + s->c_weight[j];
          const double wi = s->c_weight[i] / tw;
          const double wj = s->c_weight[j] / tw;
          const double c = wi * s->c_center[i] + wj * s->c_center[j];
          const double a = wi * s->c_alpha[i] + wj * s->c_alpha[j];
          s->c_center[i] = c;
          s->c_alpha[i] = a;
          s->c_weight[i] = tw;
          for (int k = j; k + 1 < s->n_clusters; ++k) {
            s->c_center[k] = s->c_center[k + 1];
            s->c_alpha[k] = s->c_alpha[k + 1];
            s->c_weight[k] = s->c_weight[k + 1];
          }
          s->n_clusters -= 1;
          merged = 1;
          break;
        }
      }
    }
  }
}

/* GridSpec::enforce_monotonicity, src/pde/core/grid.hpp:240-262. */
static void enforce_monotonicity(double* p, int64_t n, double x_min, double x_max) {
  if (n < 2) return;
  const double min_spacing = (x_max - x_min) / (double)(n * 100);
  p[0] = x_min;
  p[n - 1] = x_max;
  for (int64_t i = 1; i < n - 1; ++i)
    if (p[i] <= p[i - 1] + min_spacing) p[i] = p[i - 1] + min_spacing;
  for (int64_t i = n - 2; i > 0; --i)
    if (p[i] >= p[i + 1] - min_spacing) p[i] = p[i + 1] - min_spacing;
}

int32_t mo_generate_grid(const mo_grid_spec* s, double* x) {
  const int64_t n = s->n_points;
  const double xmin = s->x_min, xmax = s->x_max;
  switch (s->type) {
    case 0: { /* Uniform, grid.hpp:368-374 */
      const double dx = (xmax - xmin) / (double)(n - 1);
      for (int64_t i = 0; i < n; ++i) x[i] = xmin + (double)i * dx;
      return 0;
    }
    case 1: { /* LogSpaced, grid.hpp:376-384 */
      const double lmin = log(xmin), lmax = log(xmax);
      const double dl = (lmax - lmin) / (double)(n - 1);
      for (int64_t i = 0; i < n; ++i) x[i] = exp(lmin + (double)i * dl);
      return 0;
    }
    case 2: { /* SinhSpaced, grid.hpp:386-399 */
      const double c = s->concentration;
      const double shc = sinh(c / 2.0);
      for (int64_t i = 0; i < n; ++i) {
        const double eta = (double)i / (double)(n - 1);
        const double st = sinh(c * (eta - 0.5)) / shc;
        const double nrm = (1.0 + st) / 2.0;
        x[i] = xmin + (xmax - xmin) * nrm;
      }
      return 0;
    }
    case 3: { /* MultiSinhSpaced, grid.hpp:401-494 */
      const double range = xmax - xmin;
      if (s->n_clusters == 1) {
        const double c = s->c_alpha[0];
        const double center = s->c_center[0];
        const double shc = sinh(c / 2.0);
        const double eta_c = (center - xmin) / range;
        const int centered = fabs(eta_c - 0.5) < 1e-10;
        if (centered) {
          for (int64_t i = 0; i < n; ++i) {
            const double eta = (double)i / (double)(n - 1);
            const double st = sinh(c * (eta - 0.5)) / shc;
            const double nrm = (1.0 + st) / 2.0;
            x[i] = xmin + range * nrm;
          }
        } else {
          const double offset = center - (xmin + xmax) / 2.0;
          for (int64_t i = 0; i < n; ++i) {
            const double eta = (double)i / (double)(n - 1);
            const double st = sinh(c * (eta - eta_c)) / shc;
            const double nrm = (1.0 + st) / 2.0;
            x[i] = xmin + range * nrm + offset;
          }
          enforce_monotonicity(x, n, xmin, xmax);
        }
        return 0;
      }
      double total = 0.0;
      for (int k = 0; k < s->n_clusters; ++k) total += s->c_weight[k];
      for (int64_t i = 0; i < n; ++i) {
        const double eta = (double)i / (double)(n - 1);
        double wx = 0.0;
        for (int k = 0; k < s->n_clusters; ++k) {
          const double c = s->c_alpha[k];
          const double center = s->c_center[k];
          const double w = s->c_weight[k] / total;
          const double shc = sinh(c / 2.0);
          const double eta_c = (center - xmin) / range;
          const double st = sinh(c * (eta - eta_c)) / shc;
          const double nrm = (1.0 + st) / 2.0;
          const double offset = center - (xmin + xmax) / 2.0;
          const double xi = xmin + range * nrm + offset;
          wx += w * xi;
        }
        x[i] = wx;
      }
      enforce_monotonicity(x, n, xmin, xmax);
      return 0;
    }
  }
  return 1;
}

int32_t mo_estimate_grid(double spot, double strike, double maturity, double sigma,
                         const mo_accuracy* acc, mo_grid_spec* spec, int64_t* n_time) {
  /* estimate_pde_grid, src/option/grid_spec_types.cpp:37-118 */
  const double sst = sigma * sqrt(maturity);
  const double x0 = log(spot / strike);
  const double x_min = x0 - acc->n_sigma * sst;
  const double x_max = x0 + acc->n_sigma * sst;
  const double dx_target = sigma * sqrt(acc->tol);
  int64_t nx = (int64_t)ceil((x_max - x_min) / dx_target);
  if (nx < acc->min_spatial_points) nx = acc->min_spatial_points;
  if (nx > acc->max_spatial_points) nx = acc->max_spatial_points;
  if (nx % 2 == 0) nx++;

  memset(spec, 0, sizeof(*spec));
  spec->n_points = nx;
  spec->x_min = x_min;
  spec->x_max = x_max;
  spec->concentration = 1.0;
  spec->n_clusters = 1;
  spec->c_center[0] = x0;
  spec->c_alpha[0] = acc->alpha;
  spec->c_weight[0] = 0.5;
  if (0.0 >= x_min && 0.0 <= x_max) {
    spec->c_center[1] = 0.0;
    spec->c_alpha[1] = acc->alpha;
    spec->c_weight[1] = 1.0;
    spec->n_clusters = 2;
  }
  /* multi_sinh_spaced validation (grid.hpp:110-160); on failure the
   * reference falls back to sinh_spaced(x_min, x_max, nx, alpha). */
  int ok = nx >= 2 && x_min < x_max;
  for (int k = 0; k < spec->n_clusters && ok; ++k)
    ok = spec->c_alpha[k] > 0 && spec->c_weight[k] > 0 && spec->c_center[k] >= x_min &&
         spec->c_center[k] <= x_max;
  if (ok) {
    spec->type = 3;
    merge_clusters(spec);
  } else {
    spec->type = 2;
    spec->n_clusters = 0;
    spec->concentration = acc->alpha;
  }

  double* pts = (double*)malloc(sizeof(double) * (size_t)nx);
  if (!pts) return 2;
  mo_generate_grid(spec, pts);
  double dx_min = pts[1] - pts[0];
  for (int64_t i = 2; i < nx; ++i) dx_min = dmin(dx_min, pts[i] - pts[i - 1]);
  free(pts);
  const double dt = acc->c_t * dx_min;
  int64_t nt = (int64_t)ceil(maturity / dt);
  if (nt > acc->max_time_steps) nt = acc->max_time_steps;
  *n_time = nt;
  return 0;
}

/* -------------------------------------------------------- linear algebra -- */

/* solve_thomas, src/math/thomas_solver.hpp:86-198 (no diagonal-dominance
 * check, singularity_tol 1e-15). */
static int thomas(const double* lower, const double* diag, const double* upper,
                  const double* rhs, double* sol, int64_t n, double* ws) {
  const double tol = 1e-15;
  if (n == 0) return 0;
  if (n == 1) {
    if (fabs(diag[0]) < tol) return 1;
    sol[0] = rhs[0] / diag[0];
    return 0;
  }
  double* cp = ws;
  double* dp = ws + n;
  if (fabs(diag[0]) < tol) return 1;
  cp[0] = upper[0] / diag[0];
  dp[0] = rhs[0] / diag[0];
  for (int64_t i = 1; i < n - 1; ++i) {
    const double denom = fma(-lower[i - 1], cp[i - 1], diag[i]);
    if (fabs(denom) < tol) return 1;
    const double inv = 1.0 / denom;
    cp[i] = upper[i] * inv;
    dp[i] = fma(-lower[i - 1], dp[i - 1], rhs[i]) * inv;
  }
  {
    const int64_t i = n - 1;
    const double denom = fma(-lower[i - 1], cp[i - 1], diag[i]);
    if (fabs(denom) < tol) return 1;
    dp[i] = fma(-lower[i - 1], dp[i - 1], rhs[i]) / denom;
  }
  sol[n - 1] = dp[n - 1];
  for (int64_t i = n - 1; i > 0; --i) sol[i - 1] = fma(-cp[i - 1], sol[i], dp[i - 1]);
  return 0;
}

int32_t mo_thomas_projected(const double* lower, const double* diag, const double* upper,
                            const double* rhs, const double* psi, double* sol, int64_t n,
                            double* ws) {
  /* solve_thomas_projected, src/math/thomas_solver.hpp:321-420 */
  const double tol = 1e-15;
  if (n == 0) return 0;
  if (n == 1) {
    if (fabs(diag[0]) < tol) return 1;
    sol[0] = dmax(rhs[0] / diag[0], psi[0]);
    return 0;
  }
  double* cp = ws;
  double* dp = ws + n;
  if (fabs(diag[0]) < tol) return 1;
  cp[0] = upper[0] / diag[0];
  dp[0] = rhs[0] / diag[0];
  for (int64_t i = 1; i < n - 1; ++i) {
    const double denom = fma(-lower[i - 1], cp[i - 1], diag[i]);
    if (fabs(denom) < tol) return 1;
    const double inv = 1.0 / denom;
    cp[i] = upper[i] * inv;
    dp[i] = fma(-lower[i - 1], dp[i - 1], rhs[i]) * inv;
  }
  {
    const int64_t i = n - 1;
    const double denom = fma(-lower[i - 1], cp[i - 1], diag[i]);
    if (fabs(denom) < tol) return 1;
    dp[i] = fma(-lower[i - 1], dp[i - 1], rhs[i]) / denom;
  }
  sol[n - 1] = dmax(dp[n - 1], psi[n - 1]);
  for (int64_t i = n - 1; i > 0; --i) {
    const double unc = fma(-cp[i - 1], sol[i], dp[i - 1]);
    sol[i - 1] = dmax(unc, psi[i - 1]);
  }
  return 0;
}

/* ------------------------------------------------------------- splines -- */

typedef struct {
  int64_t n;
  const double* x;
  double *a, *b, *c, *d, *h;
} spline_t;

/* CubicSpline::build natural (src/math/cubic_spline_solver.hpp:74-170,
 * 264-369); storage is one malloc of 5n doubles plus 6n of workspace. */
static int spline_build(spline_t* s, const double* x, const double* y, int64_t n) {
  s->n = n;
  s->x = x;
  double* mem = (double*)calloc((size_t)(11 * n + 8), sizeof(double));
  if (!mem) return 2;
  s->a = mem;
  s->b = mem + n;
  s->c = mem + 2 * n;
  s->d = mem + 3 * n;
  s->h = mem + 4 * n;
  double* tl = mem + 5 * n;
  double* td = mem + 6 * n;
  double* tu = mem + 7 * n;
  double* tr = mem + 8 * n;
  double* ts = mem + 9 * n;
  double* tw = mem + 10 * n; /* needs 2m <= 2n: uses tw and beyond (calloc'd) */
  for (int64_t i = 1; i < n; ++i)
    if (x[i] <= x[i - 1]) return 1;
  const int64_t ni = n - 1;
  for (int64_t i = 0; i < ni; ++i) s->h[i] = x[i + 1] - x[i];
  s->c[0] = 0.0;
  s->c[n - 1] = 0.0;
  if (n > 2) {
    const int64_t m = n - 2;
    for (int64_t i = 0; i < m; ++i) {
      const int64_t k = i + 1;
      td[i] = 2.0 * (s->h[k - 1] + s->h[k]);
      if (i > 0) tl[i - 1] = s->h[k - 1];
      if (i < m - 1) tu[i] = s->h[k];
      const double sr = (y[k + 1] - y[k]) / s->h[k];
      const double sl = (y[k] - y[k - 1]) / s->h[k - 1];
      tr[i] = 3.0 * (sr - sl);
    }
    /* workspace of 2m: tw spans [10n, 11n+8) which holds 2m <= 2n-4 doubles
     * only when n+8 >= 2m; use a private buffer instead to stay general. */
    double* w2 = (double*)malloc(sizeof(double) * (size_t)(2 * m));
    (void)tw;
    if (!w2) return 2;
    const int bad = thomas(tl, td, tu, tr, ts, m, w2);
    free(w2);
    if (bad) return 1;
    for (int64_t i = 0; i < m; ++i) s->c[i + 1] = ts[i];
  }
  for (int64_t i = 0; i < ni; ++i) {
    s->a[i] = y[i];
    s->b[i] = (y[i + 1] - y[i]) / s->h[i] - s->h[i] * (2.0 * s->c[i] + s->c[i + 1]) / 3.0;
    s->d[i] = (s->c[i + 1] - s->c[i]) / (3.0 * s->h[i]);
  }
  return 0;
}

static void spline_free(spline_t* s) { free(s->a); }

/* find_interval, cubic_spline_solver.hpp:348-368 (lower_bound semantics). */
static int64_t spline_interval(const spline_t* s, double xe) {
  const int64_t n = s->n;
  if (xe <= s->x[0]) return 0;
  if (xe >= s->x[n - 1]) return n - 2;
  int64_t lo = 0, hi = n; /* first index with x[idx] >= xe */
  while (lo < hi) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (s->x[mid] < xe) lo = mid + 1; else hi = mid;
  }
  int64_t idx = lo;
  if (idx > 0 && (idx == n || s->x[idx] > xe)) --idx;
  return idx < n - 2 ? idx : n - 2;
}

static double spline_eval(const spline_t* s, double xe) {
  if (s->n == 1) return s->a[0];
  const int64_t i = spline_interval(s, xe);
  const double dx = xe - s->x[i];
  return s->a[i] + s->b[i] * dx + s->c[i] * (dx * dx) + s->d[i] * (dx * dx * dx);
}

static double spline_deriv(const spline_t* s, double xe) {
  if (s->n == 1) return 0.0;
  const int64_t i = spline_interval(s, xe);
  const double dx = xe - s->x[i];
  return s->b[i] + 2.0 * s->c[i] * dx + 3.0 * s->d[i] * (dx * dx);
}

int32_t mo_spline_eval(const double* x, const double* y, int64_t n, double xe,
                       double* value, double* deriv) {
  spline_t s;
  const int bad = spline_build(&s, x, y, n);
  if (bad) { spline_free(&s); return bad; }
  *value = spline_eval(&s, xe);
  *deriv = spline_deriv(&s, xe);
  spline_free(&s);
  return 0;
}

/* ------------------------------------------------------------ operator -- */

typedef struct {
  int64_t n;
  const double* x;
  int uniform;
  double dx_inv, dx_inv_sq;                 /* UniformSpacing, grid.hpp:505-520 */
  double *dxl_inv, *dxr_inv, *dxc_inv, *wl, *wr; /* NonUniformSpacing, grid.hpp:534-602 */
  double hss, q, r;                         /* BlackScholesPDE, black_scholes_pde.hpp:45-110 */
} op_t;

/* GridSpacing::compute_spacing, src/pde/core/grid.hpp:680-711. */
static int op_init(op_t* o, const double* x, int64_t n, double sigma, double r, double q) {
  memset(o, 0, sizeof(*o));
  o->n = n;
  o->x = x;
  o->hss = 0.5 * sigma * sigma;
  o->r = r;
  o->q = q;
  const double expected = (x[n - 1] - x[0]) / (double)(n - 1);
  const double tol = 100.0 * DBL_EPSILON;
  o->uniform = 1;
  for (int64_t i = 1; i < n; ++i)
    if (fabs((x[i] - x[i - 1]) - expected) > tol) { o->uniform = 0; break; }
  if (o->uniform) {
    o->dx_inv = 1.0 / expected;
    o->dx_inv_sq = o->dx_inv * o->dx_inv;
    return 0;
  }
  double* mem = (double*)malloc(sizeof(double) * (size_t)(5 * n));
  if (!mem) return 2;
  o->dxl_inv = mem;
  o->dxr_inv = mem + n;
  o->dxc_inv = mem + 2 * n;
  o->wl = mem + 3 * n;
  o->wr = mem + 4 * n;
  for (int64_t i = 1; i <= n - 2; ++i) {
    const double dl = x[i] - x[i - 1];
    const double dr = x[i + 1] - x[i];
    const double dc = 0.5 * (dl + dr);
    const int64_t k = i - 1;
    o->dxl_inv[k] = 1.0 / dl;
    o->dxr_inv[k] = 1.0 / dr;
    o->dxc_inv[k] = 1.0 / dc;
    o->wl[k] = dr / (dl + dr);
    o->wr[k] = dl / (dl + dr);
  }
  return 0;
}

static void op_free(op_t* o) { free(o->dxl_inv); }

/* CenteredDifference first/second derivative over rows [start, end)
 * (src/pde/operators/centered_difference.hpp:24-99). */
static void op_derivs(const op_t* o, const double* u, double* d2u, double* du,
                      int64_t start, int64_t end) {
  if (o->uniform) {
    const double dx2 = o->dx_inv_sq;
    const double hdx = o->dx_inv * 0.5;
    for (int64_t i = start; i < end; ++i) {
      d2u[i] = fma(u[i + 1] + u[i - 1], dx2, -2.0 * u[i] * dx2);
      du[i] = (u[i + 1] - u[i - 1]) * hdx;
    }
    return;
  }
  for (int64_t i = start; i < end; ++i) {
    const double li = o->dxl_inv[i - 1], ri = o->dxr_inv[i - 1], ci = o->dxc_inv[i - 1];
    const double fwd = (u[i + 1] - u[i]) * ri;
    const double bwd = (u[i] - u[i - 1]) * li;
    d2u[i] = (fwd - bwd) * ci;
    const double t1 = o->wl[i - 1] * (u[i] - u[i - 1]) * li;
    const double t2 = o->wr[i - 1] * (u[i + 1] - u[i]) * ri;
    du[i] = t1 + t2;
  }
}

/* apply_spatial_operator (pde_solver.hpp:322-335) -> SpatialOperator::
 * apply_interior (spatial_operator.hpp:74-97) -> BlackScholesPDE::operator()
 * (black_scholes_pde.hpp:72-76); boundary entries zeroed. */
static void op_apply(const op_t* o, const double* u, double* Lu, double* d2u, double* du) {
  const int64_t n = o->n;
  for (int64_t i = 1; i < n - 1; ++i) { d2u[i] = 0.0; du[i] = 0.0; }
  op_derivs(o, u, d2u, du, 1, n - 1);
  const double drift = o->r - o->q - o->hss;
  for (int64_t i = 1; i < n - 1; ++i) Lu[i] = o->hss * d2u[i] + drift * du[i] - o->r * u[i];
  Lu[0] = 0.0;
  Lu[n - 1] = 0.0;
}

/* assemble_jacobian (spatial_operator.hpp:123-163) and the Dirichlet
 * boundary rows (pde_solver.hpp:924-972). */
static void op_jacobian(const op_t* o, double coeff_dt, double* lower, double* diag,
                        double* upper) {
  const int64_t n = o->n;
  const double* g = o->x;
  const double a = o->hss;
  const double b = o->r - o->q - o->hss;
  const double c = -o->r;
  for (int64_t i = 1; i < n - 1; ++i) {
    const double dxl = g[i] - g[i - 1];
    const double dxr = g[i + 1] - g[i];
    const double dxa = (dxl + dxr) / 2.0;
    const double d2m = a / (dxl * dxa);
    const double d2i = -a * (1.0 / dxl + 1.0 / dxr) / dxa;
    const double d2p = a / (dxr * dxa);
    const double d1d = dxl + dxr;
    const double d1m = -b * dxr / (dxl * d1d);
    const double d1i = b * (dxr - dxl) / (dxl * dxr);
    const double d1p = b * dxl / (dxr * d1d);
    const double jl = d2m + d1m;
    const double jd = d2i + d1i + c;
    const double ju = d2p + d1p;
    lower[i - 1] = -coeff_dt * jl;
    diag[i] = 1.0 - coeff_dt * jd;
    upper[i] = -coeff_dt * ju;
  }
  diag[0] = 1.0;
  upper[0] = 0.0;
  diag[n - 1] = 1.0;
  lower[n - 2] = 0.0;
}

/* --------------------------------------------------------------- march -- */

typedef struct {
  op_t op;
  int is_put;
  double r;
  const double* x;
  int64_t n;
  double *psi, *lower, *diag, *upper, *rhs, *lpsi, *ws, *lu, *d2u, *du;
} march_t;

/* Boundary values: AmericanPutSolver / AmericanCallSolver BC functors
 * (src/option/american_option.cpp:192-210, 276-296). */
static double bc_left(const march_t* m, double t) {
  (void)t;
  return m->is_put ? dmax(1.0 - exp(m->x[0]), 0.0) : 0.0;
}
static double bc_right(const march_t* m, double t) {
  return m->is_put ? 0.0 : exp(m->x[m->n - 1]) - exp(-m->r * t);
}

static void apply_bc(const march_t* m, double* u, double t) {
  u[0] = bc_left(m, t);
  u[m->n - 1] = bc_right(m, t);
}

/* solve_implicit_stage_projected, src/pde/internal/pde_solver.hpp:525-729. */
static int stage_projected(march_t* m, double t, double coeff_dt, double* u,
                           const double* rhs_in) {
  const int64_t n = m->n;
  apply_bc(m, u, t);
  op_jacobian(&m->op, coeff_dt, m->lower, m->diag, m->upper);
  memcpy(m->rhs, rhs_in, sizeof(double) * (size_t)n);
  m->rhs[0] = bc_left(m, t);
  m->rhs[n - 1] = bc_right(m, t);
  const double* psi = m->psi;
  double psi_max = psi[0];
  for (int64_t i = 1; i < n; ++i) if (psi_max < psi[i]) psi_max = psi[i];
  if (psi_max > 0.0) {
    const double thr = 0.95 * psi_max;
    int64_t first = n - 1;
    for (int64_t i = 1; i < n - 1; ++i)
      if (psi[i] > thr && u[i] - psi[i] < 1e-8) { first = i; break; }
    if (first < n - 1) {
      op_apply(&m->op, psi, m->lpsi, m->d2u, m->du);
      for (int64_t i = first; i < n - 1; ++i) {
        if (psi[i] > thr && u[i] - psi[i] < 1e-8 && m->lpsi[i] < 0.0) {
          m->lower[i - 1] = 0.0;
          m->diag[i] = 1.0;
          m->upper[i] = 0.0;
          m->rhs[i] = psi[i];
        }
      }
    }
  }
  if (mo_thomas_projected(m->lower, m->diag, m->upper, m->rhs, psi, u, n, m->ws)) return 5;
  apply_bc(m, u, t);
  return 0;
}

int32_t mo_price_on_grid(double spot, double strike, double maturity, double sigma,
                         double rate, double q, int32_t is_put, const double* x,
                         int64_t n, int64_t nt, int32_t rannacher, double* out4,
                         double* u_final, double* u_prev_out) {
  /* validate_pricing_params, src/option/option_spec.cpp:8-40, 117-157 */
  if (!(spot > 0.0) || !isfinite(spot) || !(strike > 0.0) || !isfinite(strike) ||
      !(maturity > 0.0) || !isfinite(maturity) || !isfinite(rate) || q < 0.0 ||
      !isfinite(q) || !(sigma > 0.0) || !isfinite(sigma) || n < 3 || nt < 1)
    return 1;
  march_t m;
  memset(&m, 0, sizeof(m));
  m.is_put = is_put;
  m.r = rate;
  m.x = x;
  m.n = n;
  if (op_init(&m.op, x, n, sigma, rate, q)) return 2;
  double* mem = (double*)calloc((size_t)(14 * n), sizeof(double));
  if (!mem) { op_free(&m.op); return 2; }
  m.psi = mem;
  m.lower = mem + n;
  m.diag = mem + 2 * n;
  m.upper = mem + 3 * n;
  m.rhs = mem + 4 * n;
  m.lpsi = mem + 5 * n;
  m.ws = mem + 6 * n; /* 2n */
  m.lu = mem + 8 * n;
  m.d2u = mem + 9 * n;
  m.du = mem + 10 * n;
  double* u = mem + 11 * n;
  double* up = mem + 12 * n;
  double* rhs = mem + 13 * n;

  /* payoff = obstacle: log_put_payoff / log_call_payoff (option_spec.hpp:122-135) */
  for (int64_t i = 0; i < n; ++i)
    m.psi[i] = is_put ? dmax(1.0 - exp(x[i]), 0.0) : dmax(exp(x[i]) - 1.0, 0.0);

  /* PDESolver::initialize, pde_solver.hpp:96-109 */
  for (int64_t i = 0; i < n; ++i) u[i] = m.psi[i];
  apply_bc(&m, u, 0.0);
  for (int64_t i = 0; i < n; ++i) u[i] = dmax(u[i], m.psi[i]);
  memcpy(up, u, sizeof(double) * (size_t)n);

  /* TimeDomain::from_n_steps (time_domain.hpp:36-45); time_points i*dt */
  const double dt = (maturity - 0.0) / (double)nt;
  const double gamma = 2.0 - sqrt(2.0); /* TRBDF2Config, trbdf2_config.hpp:20 */
  int rc = 0;
  double t = 0.0;
  int64_t step = 0;
  /* PDESolver::solve, pde_solver.hpp:114-178; Rannacher 413-447 */
  if (rannacher && nt > 0) {
    const double half = 0.5 * dt;
    const double t_mid = t + half;
    const double t_next = t + dt;
    memcpy(up, u, sizeof(double) * (size_t)n);
    memcpy(rhs, up, sizeof(double) * (size_t)n);
    memcpy(u, up, sizeof(double) * (size_t)n);
    rc = stage_projected(&m, t_mid, half, u, rhs);
    if (!rc) {
      memcpy(up, u, sizeof(double) * (size_t)n);
      memcpy(rhs, up, sizeof(double) * (size_t)n);
      memcpy(u, up, sizeof(double) * (size_t)n);
      rc = stage_projected(&m, t_next, half, u, rhs);
    }
    t = 0.0 + 1.0 * dt;
    step = 1;
  }
  for (; !rc && step < nt; ++step) {
    const double t_next = 0.0 + (double)(step + 1) * dt;
    memcpy(up, u, sizeof(double) * (size_t)n);
    /* solve_stage1, pde_solver.hpp:342-362 */
    const double t1 = t + gamma * dt;
    const double w1 = gamma * dt / 2.0;
    op_apply(&m.op, up, m.lu, m.d2u, m.du);
    for (int64_t i = 0; i < n; ++i) rhs[i] = fma(w1, m.lu[i], up[i]);
    memcpy(u, up, sizeof(double) * (size_t)n);
    rc = stage_projected(&m, t1, w1, u, rhs);
    if (rc) break;
    /* solve_stage2, pde_solver.hpp:370-395 */
    const double omg = 1.0 - gamma;
    const double tmg = 2.0 - gamma;
    const double den = gamma * tmg;
    const double alpha = 1.0 / den;
    const double beta = -(omg * omg) / den;
    const double w2 = (1.0 - gamma) * dt / (2.0 - gamma);
    for (int64_t i = 0; i < n; ++i) rhs[i] = fma(alpha, u[i], beta * up[i]);
    rc = stage_projected(&m, t_next, w2, u, rhs);
    t = t_next;
  }

  if (!rc) {
    /* AmericanOptionResult, src/option/american_option_result.cpp:25-121 */
    spline_t sp, spp;
    const double xs = log(spot / strike);
    int bad = spline_build(&sp, x, u, n);
    bad |= spline_build(&spp, x, up, n);
    if (bad) rc = 5;
    if (!rc) {
      double value;
      if (xs <= x[0]) value = u[0] * strike;
      else if (xs >= x[n - 1]) value = u[n - 1] * strike;
      else value = dmax(0.0, spline_eval(&sp, xs)) * strike;
      const double delta = spline_deriv(&sp, xs) * (strike / spot);
      /* gamma: stencil derivatives on rows [1, n-2), linear interpolation */
      double* dv = (double*)calloc((size_t)(2 * n), sizeof(double));
      double* d2v = dv + n;
      op_derivs(&m.op, u, d2v, dv, 1, n - 2);
      int64_t il, ir;
      if (xs <= x[0]) { il = ir = 0; }
      else if (xs >= x[n - 1]) { il = ir = n - 1; }
      else {
        int64_t lo = 0, hi = n;
        while (lo < hi) {
          const int64_t mid = lo + (hi - lo) / 2;
          if (x[mid] < xs) lo = mid + 1; else hi = mid;
        }
        ir = lo;
        il = ir > 0 ? ir - 1 : 0;
        if (fabs(x[ir] - xs) < 1e-14) il = ir;
      }
      double d1, d2;
      if (il == ir) { d1 = dv[il]; d2 = d2v[il]; }
      else {
        const double al = (xs - x[il]) / (x[ir] - x[il]);
        d1 = dv[il] + al * (dv[ir] - dv[il]);
        d2 = d2v[il] + al * (d2v[ir] - d2v[il]);
      }
      free(dv);
      const double kos2 = strike / (spot * spot);
      const double gam = fma(kos2, d2, -kos2 * d1);
      const double vc = spline_eval(&sp, xs);
      const double vp = spline_eval(&spp, xs);
      const double theta = (vp - vc) / dt * strike;
      out4[0] = value;
      out4[1] = delta;
      out4[2] = gam;
      out4[3] = theta;
    }
    spline_free(&sp);
    spline_free(&spp);
    if (u_final) memcpy(u_final, u, sizeof(double) * (size_t)n);
    if (u_prev_out) memcpy(u_prev_out, up, sizeof(double) * (size_t)n);
  }
  free(mem);
  op_free(&m.op);
  return rc;
}

/* ---------------------------------------------------------------- batch -- */

static int32_t price_one(double S, double K, double T, double sig, double r, double q,
                         int32_t is_put, int64_t nx_req, int64_t nt_req, int32_t rannacher,
                         double grid_sigma, double* out4, int64_t* dims) {
  mo_accuracy acc;
  mo_default_accuracy(&acc);
  if (nx_req > 0) {
    acc.min_spatial_points = nx_req;
    acc.max_spatial_points = nx_req;
  }
  mo_grid_spec spec;
  int64_t nt_auto = 0;
  const double gs = grid_sigma > 0.0 ? grid_sigma : sig;
  if (!(S > 0.0) || !(K > 0.0) || !(T > 0.0) || !(gs > 0.0)) return 1;
  if (mo_estimate_grid(S, K, T, gs, &acc, &spec, &nt_auto)) return 2;
  const int64_t nt = nx_req > 0 ? nt_req : nt_auto;
  double* x = (double*)malloc(sizeof(double) * (size_t)spec.n_points);
  if (!x) return 2;
  mo_generate_grid(&spec, x);
  const int32_t rc =
      mo_price_on_grid(S, K, T, sig, r, q, is_put, x, spec.n_points, nt, rannacher, out4, 0, 0);
  if (dims) { dims[0] = spec.n_points; dims[1] = nt; }
  free(x);
  return rc;
}

int32_t mo_price_batch(int64_t n, const double* S, const double* K, const double* T,
                       const double* sigma, const double* r, const double* q,
                       const int32_t* is_put, const int64_t* nx, const int64_t* nt,
                       int32_t rannacher, int32_t n_threads, double* out4,
                       int64_t* out_dims, int32_t* status) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t i = 0; i < n; ++i) {
    status[i] = price_one(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i],
                          nx ? nx[i] : 0, nt ? nt[i] : 0, rannacher, 0.0, out4 + 4 * i,
                          out_dims ? out_dims + 2 * i : 0);
  }
  (void)n_threads;
  return 0;
}

/* ----------------------------------------------------------------- IV --- */

typedef struct {
  double S, K, T, r, q, price;
  int32_t is_put;
  const double* x;
  int64_t n, nt;
} ivq_t;

/* IVSolver::objective_function (iv_solver.cpp:48-119): value_at(spot) - P. */
static double iv_objective(const ivq_t* qy, double vol) {
  double out4[4];
  if (mo_price_on_grid(qy->S, qy->K, qy->T, vol, qy->r, qy->q, qy->is_put, qy->x, qy->n,
                       qy->nt, 1, out4, 0, 0))
    return NAN;
  return out4[0] - qy->price;
}

/* brent_find_root, src/math/root_finding.hpp:145-302 (tol 1e-6, 100 iters). */
static int32_t brent(const ivq_t* qy, double a, double b, double* root, double* iters,
                     double* ferr) {
  const double tol = 1e-6;
  const int max_iter = 100;
  double fa = iv_objective(qy, a);
  double fb = iv_objective(qy, b);
  if (!isfinite(fa) || !isfinite(fb)) { *iters = 0; *ferr = NAN; return 12; }
  if (fa * fb > 0.0) { *iters = 0; *ferr = dmin(fabs(fa), fabs(fb)); return 10; }
  if (fabs(fa) < tol) { *root = a; *iters = 0; *ferr = fabs(fa); return 0; }
  if (fabs(fb) < tol) { *root = b; *iters = 0; *ferr = fabs(fb); return 0; }
  if (fabs(fa) < fabs(fb)) { double t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
  double c = a, fc = fa, d = 0.0;
  int mflag = 1;
  for (int it = 0; it < max_iter; ++it) {
    if (fabs(fb) < tol || fabs(b - a) < tol) {
      *root = b; *iters = it + 1; *ferr = fabs(fb); return 0;
    }
    double s;
    if (fa != fc && fb != fc) {
      s = a * fb * fc / ((fa - fb) * (fa - fc)) + b * fa * fc / ((fb - fa) * (fb - fc)) +
          c * fa * fb / ((fc - fa) * (fc - fb));
    } else {
      s = b - fb * (b - a) / (fb - fa);
    }
    const double bis = (3.0 * a + b) / 4.0;
    const int c1 = !((s > bis && s < b) || (s < bis && s > b));
    const int c2 = mflag && fabs(s - b) >= fabs(b - c) / 2.0;
    const int c3 = !mflag && fabs(s - b) >= fabs(c - d) / 2.0;
    const int c4 = mflag && fabs(b - c) < tol;
    const int c5 = !mflag && fabs(c - d) < tol;
    if (c1 || c2 || c3 || c4 || c5) { s = (a + b) / 2.0; mflag = 1; } else { mflag = 0; }
    const double fs = iv_objective(qy, s);
    if (!isfinite(fs)) { *root = s; *iters = it + 1; *ferr = NAN; return 12; }
    d = c;
    c = b;
    fc = fb;
    if (fa * fs < 0.0) { b = s; fb = fs; } else { a = s; fa = fs; }
    if (fabs(fa) < fabs(fb)) { double t = a; a = b; b = t; t = fa; fa = fb; fb = t; }
  }
  *root = b;
  *iters = max_iter;
  *ferr = fabs(fb);
  return 11;
}

int32_t mo_iv_batch(int64_t n, const double* S, const double* K, const double* T,
                    const double* r, const double* q, const int32_t* is_put,
                    const double* price, const double* grid_sigma, const int64_t* nx,
                    const int64_t* nt, int32_t n_threads, double* out3, int32_t* status) {
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int64_t i = 0; i < n; ++i) {
    double* o = out3 + 3 * i;
    o[0] = NAN; o[1] = 0; o[2] = NAN;
    /* validate_iv_query, option_spec.cpp:52-112 */
    const double intrinsic = is_put[i] ? dmax(K[i] - S[i], 0.0) : dmax(S[i] - K[i], 0.0);
    const double upper = is_put[i] ? K[i] : S[i];
    if (!(S[i] > 0.0) || !isfinite(S[i]) || !(K[i] > 0.0) || !isfinite(K[i]) ||
        !(T[i] > 0.0) || !isfinite(T[i]) || !isfinite(r[i]) || q[i] < 0.0 ||
        !isfinite(q[i]) || !isfinite(price[i]) || price[i] <= 0.0 ||
        price[i] < intrinsic || price[i] > upper) {
      status[i] = 1;
      continue;
    }
    mo_accuracy acc;
    mo_default_accuracy(&acc);
    acc.min_spatial_points = nx[i];
    acc.max_spatial_points = nx[i];
    mo_grid_spec spec;
    int64_t nt_auto;
    mo_estimate_grid(S[i], K[i], T[i], grid_sigma[i], &acc, &spec, &nt_auto);
    double* x = (double*)malloc(sizeof(double) * (size_t)spec.n_points);
    mo_generate_grid(&spec, x);
    ivq_t qy = {S[i], K[i], T[i], r[i], q[i], price[i], is_put[i], x, spec.n_points, nt[i]};
    /* solve_brent bracket, iv_solver.cpp:133-160 */
    const double tv_ratio = (price[i] - intrinsic) / price[i];
    const double hi = tv_ratio > 0.5 ? 3.0 : (tv_ratio > 0.2 ? 2.0 : 1.5);
    status[i] = brent(&qy, 0.01, hi, &o[0], &o[1], &o[2]);
    free(x);
  }
  (void)n_threads;
  return 0;
}

/* ------------------------------------------------------------ B-splines -- */

void mo_clamped_knots(const double* x, int64_t n, double* t) {
  /* clamped_knots_cubic, src/math/bspline/bspline_basis.hpp:47-91 */
  for (int k = 0; k < 4; ++k) t[k] = x[0];
  if (n > 4) {
    const int64_t interior = n - 4, intervals = n - 1;
    for (int64_t idx = 0; idx < interior; ++idx) {
      const double ratio = (double)(idx + 1) / (double)(interior + 1);
      const double pos = ratio * (double)intervals;
      int64_t low = (int64_t)floor(pos);
      if (low >= intervals) low = intervals - 1;
      const double frac = pos - (double)low;
      const double left = x[low], right = x[low + 1];
      double knot = (1.0 - frac) * left + frac * right;
      const double spacing = right - left;
      const double e1 = 128.0 * DBL_EPSILON * spacing;
      const double e2 = DBL_EPSILON * dmax(fabs(right), 1.0);
      const double eps = dmax(e1, e2);
      const double lo = left + eps, hi = right - eps;
      if (knot < lo) knot = lo;            /* std::clamp(v, lo, hi) */
      else if (hi < knot) knot = hi;
      t[4 + idx] = knot;
    }
  }
  for (int k = 0; k < 4; ++k) t[n + k] = x[n - 1];
}

/* find_span_cubic, bspline_basis.hpp:120-142 */
static int span_cubic(const double* t, int nk, double x) {
  const int n_ctrl = nk - 4;
  const int max_span = n_ctrl - 1 > 3 ? n_ctrl - 1 : 3;
  if (x <= t[3]) return 3;
  if (x >= t[n_ctrl]) return max_span;
  int lo = 3, hi = n_ctrl + 1; /* upper_bound: first t > x */
  while (lo < hi) {
    const int mid = lo + (hi - lo) / 2;
    if (t[mid] <= x) lo = mid + 1; else hi = mid;
  }
  int i = lo - 1;
  if (i < 3) i = 3;
  if (i > max_span) i = max_span;
  return i;
}

/* cubic_basis_nonuniform, bspline_basis.hpp:164-238 (full triangle). */
static void basis_cubic(const double* t, int n, int i, double x, double N[4]) {
  if (fabs(x - t[n - 1]) < 64.0 * DBL_EPSILON * dmax(fabs(t[n - 1]), 1.0)) {
    N[0] = 1.0; N[1] = 0.0; N[2] = 0.0; N[3] = 0.0;
    return;
  }
  double N0[4] = {0, 0, 0, 0}, N1[4] = {0, 0, 0, 0}, N2[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 1 < n) N0[k] = (t[idx] <= x && x < t[idx + 1]) ? 1.0 : 0.0;
  }
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 2 < n) {
      const double ld = t[idx + 1] - t[idx], rd = t[idx + 2] - t[idx + 1];
      const double l = (ld > 0.0) ? (x - t[idx]) / ld * N0[k] : 0.0;
      const double r = (rd > 0.0 && k > 0) ? (t[idx + 2] - x) / rd * N0[k - 1] : 0.0;
      N1[k] = l + r;
    }
  }
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 3 < n) {
      const double ld = t[idx + 2] - t[idx], rd = t[idx + 3] - t[idx + 1];
      const double l = (ld > 0.0) ? (x - t[idx]) / ld * N1[k] : 0.0;
      const double r = (rd > 0.0 && k > 0) ? (t[idx + 3] - x) / rd * N1[k - 1] : 0.0;
      N2[k] = l + r;
    }
  }
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 4 < n) {
      const double ld = t[idx + 3] - t[idx], rd = t[idx + 4] - t[idx + 1];
      const double l = (ld > 0.0) ? (x - t[idx]) / ld * N2[k] : 0.0;
      const double r = (rd > 0.0 && k > 0) ? (t[idx + 4] - x) / rd * N2[k - 1] : 0.0;
      N[k] = l + r;
    } else {
      N[k] = 0.0;
    }
  }
}

int32_t mo_bspline4d_eval(const int64_t* sizes, const double* grids, const double* coeffs,
                          const double* q, int64_t n, double* out) {
  double* knots[4];
  const double* g[4];
  int nk[4];
  const double* gp = grids;
  for (int d = 0; d < 4; ++d) {
    if (sizes[d] < 4) return 1;
    nk[d] = (int)sizes[d] + 4;
    knots[d] = (double*)malloc(sizeof(double) * (size_t)nk[d]);
    g[d] = gp;
    mo_clamped_knots(gp, sizes[d], knots[d]);
    gp += sizes[d];
  }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (int64_t qi = 0; qi < n; ++qi) {
    int span[4];
    double w[4][4];
    for (int d = 0; d < 4; ++d) {
      double x = q[4 * qi + d];
      const double lo = g[d][0], hi = g[d][sizes[d] - 1];
      if (x <= lo) x = lo;                       /* clamp_bspline_query */
      else if (x >= hi) x = nextafter(hi, -INFINITY);
      span[d] = span_cubic(knots[d], nk[d], x);
      basis_cubic(knots[d], nk[d], span[d], x, w[d]);
    }
    /* eval_tensor_product, bspline_nd.hpp:314-346 */
    double s0 = 0.0;
    for (int o0 = 0; o0 < 4; ++o0) {
      const int i0 = span[0] - o0;
      if ((unsigned)i0 >= (unsigned)sizes[0]) continue;
      double s1 = 0.0;
      for (int o1 = 0; o1 < 4; ++o1) {
        const int i1 = span[1] - o1;
        if ((unsigned)i1 >= (unsigned)sizes[1]) continue;
        double s2 = 0.0;
        for (int o2 = 0; o2 < 4; ++o2) {
          const int i2 = span[2] - o2;
          if ((unsigned)i2 >= (unsigned)sizes[2]) continue;
          double s3 = 0.0;
          for (int o3 = 0; o3 < 4; ++o3) {
            const int i3 = span[3] - o3;
            if ((unsigned)i3 >= (unsigned)sizes[3]) continue;
            const double c =
                coeffs[(((int64_t)i0 * sizes[1] + i1) * sizes[2] + i2) * sizes[3] + i3];
            s3 = fma(c, w[3][o3], s3);
          }
          s2 = fma(s3, w[2][o2], s2);
        }
        s1 = fma(s2, w[1][o1], s1);
      }
      s0 = fma(s1, w[0][o0], s0);
    }
    out[qi] = s0;
  }
  for (int d = 0; d < 4; ++d) free(knots[d]);
  return 0;
}

/* ------------------------------------------------------------- tangent -- */

/* Tangent bands of assemble_jacobian for operator coefficients (a, b, c):
 * the rows are linear in them, so these are d(A)/d(theta) for
 * (a, b, c) = (da, db, dc); boundary rows are constant (zero). */
static void tangent_bands(const double* g, int64_t n, double a, double b, double c, double w,
                          double* lower, double* diag, double* upper) {
  for (int64_t i = 1; i < n - 1; ++i) {
    const double dxl = g[i] - g[i - 1];
    const double dxr = g[i + 1] - g[i];
    const double dxa = (dxl + dxr) / 2.0;
    const double d1d = dxl + dxr;
    const double jl = a / (dxl * dxa) + (-b * dxr / (dxl * d1d));
    const double jd = (-a * (1.0 / dxl + 1.0 / dxr) / dxa) + b * (dxr - dxl) / (dxl * dxr) + c;
    const double ju = a / (dxr * dxa) + b * dxl / (dxr * d1d);
    lower[i - 1] = -w * jl;
    diag[i] = -w * jd;
    upper[i] = -w * ju;
  }
  diag[0] = 0.0;
  upper[0] = 0.0;
  diag[n - 1] = 0.0;
  lower[n - 2] = 0.0;
}

typedef struct {
  march_t m;
  op_t dop[3];                       /* the operator along each direction */
  double dbc[3];                     /* 1 where the right boundary moves (rate) */
  double *tl[3], *td[3], *tu[3], *trhs[3], *tcp[3], *tdp[3], *tw[3];
} tmarch_t;

/* One projected stage with tangents: u / tv[j] guess in, solution out. */
static int tangent_stage(tmarch_t* T, double t, double w, double* u, double** tv,
                         const double* rhs_in, double* const* trhs_in) {
  march_t* m = &T->m;
  const int64_t n = m->n;
  apply_bc(m, u, t);
  op_jacobian(&m->op, w, m->lower, m->diag, m->upper);
  memcpy(m->rhs, rhs_in, sizeof(double) * (size_t)n);
  m->rhs[0] = bc_left(m, t);
  m->rhs[n - 1] = bc_right(m, t);
  const double dbr = m->is_put ? 0.0 : t * exp(-m->r * t);
  for (int j = 0; j < 3; ++j) {
    tangent_bands(m->x, n, T->dop[j].hss, T->dop[j].r - T->dop[j].q - T->dop[j].hss, -T->dop[j].r, w,
                  T->tl[j], T->td[j], T->tu[j]);
    memcpy(T->trhs[j], trhs_in[j], sizeof(double) * (size_t)n);
    T->trhs[j][0] = 0.0;
    T->trhs[j][n - 1] = T->dbc[j] * dbr;
  }
  const double* psi = m->psi;
  double psi_max = psi[0];
  for (int64_t i = 1; i < n; ++i) if (psi_max < psi[i]) psi_max = psi[i];
  if (psi_max > 0.0) {
    const double thr = 0.95 * psi_max;
    op_apply(&m->op, psi, m->lpsi, m->d2u, m->du);
    for (int64_t i = 1; i < n - 1; ++i) {
      if (psi[i] > thr && u[i] - psi[i] < 1e-8 && m->lpsi[i] < 0.0) {
        m->lower[i - 1] = 0.0;
        m->diag[i] = 1.0;
        m->upper[i] = 0.0;
        m->rhs[i] = psi[i];
        for (int j = 0; j < 3; ++j) {
          T->tl[j][i - 1] = 0.0;
          T->td[j][i] = 0.0;
          T->tu[j][i] = 0.0;
          T->trhs[j][i] = 0.0;
        }
      }
    }
  }
  /* projected Thomas and its tangent */
  double* cp = m->ws;
  double* dp = m->ws + n;
  const double* lo = m->lower;
  const double* di = m->diag;
  const double* up = m->upper;
  const double* r = m->rhs;
  if (fabs(di[0]) < 1e-15) return 5;
  cp[0] = up[0] / di[0];
  dp[0] = r[0] / di[0];
  for (int j = 0; j < 3; ++j) {
    T->tcp[j][0] = (T->tu[j][0] - cp[0] * T->td[j][0]) / di[0];
    T->tdp[j][0] = (T->trhs[j][0] - dp[0] * T->td[j][0]) / di[0];
  }
  for (int64_t i = 1; i < n; ++i) {
    const double denom = fma(-lo[i - 1], cp[i - 1], di[i]);
    if (fabs(denom) < 1e-15) return 5;
    const double num = fma(-lo[i - 1], dp[i - 1], r[i]);
    for (int j = 0; j < 3; ++j) {
      const double tden = T->td[j][i] - T->tl[j][i - 1] * cp[i - 1] - lo[i - 1] * T->tcp[j][i - 1];
      const double tnum = T->trhs[j][i] - T->tl[j][i - 1] * dp[i - 1] - lo[i - 1] * T->tdp[j][i - 1];
      T->tdp[j][i] = (tnum - num / denom * tden) / denom;
      if (i < n - 1) T->tcp[j][i] = (T->tu[j][i] - up[i] / denom * tden) / denom;
    }
    if (i < n - 1) {
      const double inv = 1.0 / denom;
      cp[i] = up[i] * inv;
      dp[i] = num * inv;
    } else {
      dp[i] = num / denom;
    }
  }
  double x = dmax(dp[n - 1], psi[n - 1]);
  for (int j = 0; j < 3; ++j) tv[j][n - 1] = dp[n - 1] < psi[n - 1] ? 0.0 : T->tdp[j][n - 1];
  u[n - 1] = x;
  for (int64_t i = n - 1; i > 0; --i) {
    const double unc = fma(-cp[i - 1], u[i], dp[i - 1]);
    const int act = unc < psi[i - 1];
    for (int j = 0; j < 3; ++j)
      tv[j][i - 1] = act ? 0.0 : T->tdp[j][i - 1] - T->tcp[j][i - 1] * u[i] - cp[i - 1] * tv[j][i];
    u[i - 1] = dmax(unc, psi[i - 1]);
  }
  apply_bc(m, u, t);
  for (int j = 0; j < 3; ++j) {
    tv[j][0] = 0.0;
    tv[j][n - 1] = T->dbc[j] * dbr;
  }
  return 0;
}

int32_t mo_price_tangent_on_grid(double spot, double strike, double maturity, double sigma,
                                 double rate, double q, int32_t is_put, const double* x,
                                 int64_t n, int64_t nt, double* out6) {
  if (!(spot > 0.0) || !isfinite(spot) || !(strike > 0.0) || !isfinite(strike) ||
      !(maturity > 0.0) || !isfinite(maturity) || !isfinite(rate) || q < 0.0 ||
      !isfinite(q) || !(sigma > 0.0) || !isfinite(sigma) || n < 3 || nt < 1)
    return 1;
  tmarch_t T;
  memset(&T, 0, sizeof(T));
  march_t* m = &T.m;
  m->is_put = is_put;
  m->r = rate;
  m->x = x;
  m->n = n;
  if (op_init(&m->op, x, n, sigma, rate, q)) return 2;
  /* direction operators: (a, b, c) -> (da, db, dc) with b = r - q - a, c = -r */
  const double da[3] = {sigma, 0.0, 0.0}, db[3] = {-sigma, 1.0, -1.0}, dc[3] = {0.0, -1.0, 0.0};
  for (int j = 0; j < 3; ++j) {
    T.dop[j] = m->op;
    T.dop[j].hss = da[j];
    T.dop[j].r = -dc[j];
    T.dop[j].q = -dc[j] - da[j] - db[j];
    T.dbc[j] = j == 1 ? 1.0 : 0.0;
  }
  const size_t nn = (size_t)n;
  double* mem = (double*)calloc(nn * (14 + 3 * 9 + 1), sizeof(double));
  if (!mem) { op_free(&m->op); return 2; }
  m->psi = mem;
  m->lower = mem + n;
  m->diag = mem + 2 * n;
  m->upper = mem + 3 * n;
  m->rhs = mem + 4 * n;
  m->lpsi = mem + 5 * n;
  m->ws = mem + 6 * n;
  m->lu = mem + 8 * n;
  m->d2u = mem + 9 * n;
  m->du = mem + 10 * n;
  double* u = mem + 11 * n;
  double* up = mem + 12 * n;
  double* rhs = mem + 13 * n;
  double* base = mem + 14 * n;
  double *tv[3], *tvp[3], *trhs[3];
  for (int j = 0; j < 3; ++j) {
    double* b = base + (size_t)j * 9 * nn;
    T.tl[j] = b; T.td[j] = b + n; T.tu[j] = b + 2 * n; T.trhs[j] = b + 3 * n;
    T.tcp[j] = b + 4 * n; T.tdp[j] = b + 5 * n;
    tv[j] = b + 6 * n; tvp[j] = b + 7 * n; trhs[j] = b + 8 * n;
  }
  double* tmp = base + 27 * nn;
  for (int64_t i = 0; i < n; ++i)
    m->psi[i] = is_put ? dmax(1.0 - exp(x[i]), 0.0) : dmax(exp(x[i]) - 1.0, 0.0);
  for (int64_t i = 0; i < n; ++i) u[i] = m->psi[i];
  apply_bc(m, u, 0.0);
  for (int64_t i = 0; i < n; ++i) u[i] = dmax(u[i], m->psi[i]);
  const double dt = maturity / (double)nt;
  const double gamma = 2.0 - sqrt(2.0);
  int rc = 0;
  const double half = 0.5 * dt;
  for (int hs = 0; hs < 2 && !rc; ++hs) {
    memcpy(rhs, u, sizeof(double) * nn);
    for (int j = 0; j < 3; ++j) memcpy(trhs[j], tv[j], sizeof(double) * nn);
    rc = tangent_stage(&T, hs == 0 ? half : dt, half, u, tv, rhs, trhs);
  }
  double t = dt;
  for (int64_t step = 1; !rc && step < nt; ++step) {
    const double t_next = (double)(step + 1) * dt;
    memcpy(up, u, sizeof(double) * nn);
    for (int j = 0; j < 3; ++j) memcpy(tvp[j], tv[j], sizeof(double) * nn);
    const double w1 = gamma * dt / 2.0;
    op_apply(&m->op, up, m->lu, m->d2u, m->du);
    for (int64_t i = 0; i < n; ++i) rhs[i] = fma(w1, m->lu[i], up[i]);
    for (int j = 0; j < 3; ++j) {
      op_apply(&T.dop[j], up, tmp, m->d2u, m->du);           /* dL(u) */
      op_apply(&m->op, tvp[j], m->lu, m->d2u, m->du);         /* L(du) */
      for (int64_t i = 0; i < n; ++i) trhs[j][i] = w1 * (tmp[i] + m->lu[i]) + tvp[j][i];
    }
    rc = tangent_stage(&T, t + gamma * dt, w1, u, tv, rhs, trhs);
    if (rc) break;
    const double omg = 1.0 - gamma, tmg = 2.0 - gamma, den = gamma * tmg;
    const double alpha = 1.0 / den, beta = -(omg * omg) / den;
    const double w2 = (1.0 - gamma) * dt / (2.0 - gamma);
    for (int64_t i = 0; i < n; ++i) rhs[i] = fma(alpha, u[i], beta * up[i]);
    for (int j = 0; j < 3; ++j)
      for (int64_t i = 0; i < n; ++i) trhs[j][i] = alpha * tv[j][i] + beta * tvp[j][i];
    rc = tangent_stage(&T, t_next, w2, u, tv, rhs, trhs);
    t = t_next;
  }
  if (!rc) {
    const double xs = log(spot / strike);
    spline_t sp;
    if (spline_build(&sp, x, u, n)) rc = 5;
    if (!rc) {
      const double s = spline_eval(&sp, xs), sd = spline_deriv(&sp, xs);
      double tvv[3];
      for (int j = 0; j < 3 && !rc; ++j) {
        spline_t st;
        if (spline_build(&st, x, tv[j], n)) rc = 5;
        else tvv[j] = spline_eval(&st, xs);
        spline_free(&st);
      }
      if (!rc) {
        double value, dK;
        if (xs <= x[0] || xs >= x[n - 1]) {
          const int64_t e = xs <= x[0] ? 0 : n - 1;
          value = u[e] * strike;
          for (int j = 0; j < 3; ++j) tvv[j] = tv[j][e];
          dK = u[e];
        } else {
          const int pos = 0.0 < s;
          value = (pos ? s : 0.0) * strike;
          for (int j = 0; j < 3; ++j) tvv[j] = pos ? tvv[j] : 0.0;
          dK = pos ? s - sd : 0.0;
        }
        out6[0] = value;
        out6[1] = sd * (strike / spot);
        out6[2] = tvv[0] * strike;
        out6[3] = tvv[1] * strike;
        out6[4] = tvv[2] * strike;
        out6[5] = dK;
      }
    }
    spline_free(&sp);
  }
  free(mem);
  op_free(&m->op);
  return rc;
}
