// Test infrastructure only: a thin extern "C" driver over the UNMODIFIED
// reference C++ sources (compiled from the reference tree by oracle/ref/Makefile
// into oracle/_ref/).  It exists to (a) generate golden vectors for tests/golden
// and (b) pin the C restatement in oracle/mango_oracle.c.  Nothing in the
// product links or loads this library.
//
// Grid rule used by the fixed-size paths (BASELINE configs 0/1/3/4): the
// spatial GridSpec comes from estimate_pde_grid with
// min_spatial_points == max_spatial_points == nx
// (src/option/grid_spec_types.cpp:37-118), and the time axis from
// PDEGridConfig{spec, nt} (src/option/grid_spec_types.hpp:55-59).
#include "mango/option/american_option.hpp"
#include "mango/option/yield_curve.hpp"
#include "mango/support/crc64.hpp"
#include "mango/option/american_option_batch.hpp"
#include "mango/option/iv_solver.hpp"
#include "mango/option/grid_spec_types.hpp"
#include "mango/math/bspline/bspline_nd.hpp"
#include "mango/math/bspline/bspline_basis.hpp"
#include "mango/option/table/bspline/bspline_builder.hpp"
#include "mango/option/table/bspline/bspline_surface.hpp"
#include "mango/option/table/bspline/bspline_tensor_accessor.hpp"
#include "mango/option/table/eep/eep_decomposer.hpp"
#include "mango/option/interpolated_iv_solver.hpp"

#include <omp.h>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <array>

using namespace mango;

// The reference declares this friend for its tests (bspline_builder.hpp:368);
// the oracle defines its own to reach the private sweep stage.
namespace mango::testing {
template <>
struct PriceTableBuilderAccess<4> {
  static BatchAmericanOptionResult solve_batch(const PriceTableBuilderND<4>& b,
                                               const std::vector<PricingParams>& batch,
                                               const PriceTableAxesND<4>& a) {
    return b.solve_batch(batch, a);
  }
};
}  // namespace mango::testing

namespace {

PricingParams make_params(double S, double K, double T, double sigma, double r,
                          double q, int32_t is_put) {
  PricingParams p;
  p.spot = S;
  p.strike = K;
  p.maturity = T;
  p.volatility = sigma;
  p.rate = r;
  p.dividend_yield = q;
  p.option_type = is_put ? OptionType::PUT : OptionType::CALL;
  return p;
}

// nx == 0 -> reference auto grid (GridAccuracyParams{}); else grid rule above.
std::optional<PDEGridSpec> grid_for(const PricingParams& p, int64_t nx, int64_t nt,
                                    double grid_sigma) {
  if (nx <= 0) return std::nullopt;
  GridAccuracyParams acc;
  acc.min_spatial_points = static_cast<size_t>(nx);
  acc.max_spatial_points = static_cast<size_t>(nx);
  PricingParams pg = p;
  if (grid_sigma > 0.0) pg.volatility = grid_sigma;
  auto [spec, td] = estimate_pde_grid(pg, acc);
  (void)td;
  return PDEGridSpec{PDEGridConfig{spec, static_cast<size_t>(nt), {}}};
}

}  // namespace

extern "C" {

// Price n options through AmericanOptionSolver::create + solve, OpenMP over
// options exactly like solve_regular_batch's loop body
// (src/option/american_option_batch.cpp:442-511).
// out4 = [value, delta, gamma, theta] per option; out_dims = [nx, nt].
int32_t ref_price_batch(int64_t n, const double* S, const double* K, const double* T,
                        const double* sigma, const double* r, const double* q,
                        const int32_t* is_put, const int64_t* nx, const int64_t* nt,
                        int32_t rannacher, int32_t n_threads, double* out4,
                        int64_t* out_dims, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    auto p = make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]);
    auto grid = grid_for(p, nx ? nx[i] : 0, nt ? nt[i] : 0, 0.0);
    auto solver = AmericanOptionSolver::create(p, grid);
    if (!solver) { status[i] = 1; continue; }
    TRBDF2Config cfg;
    cfg.rannacher_startup = rannacher != 0;
    solver->set_trbdf2_config(cfg);
    auto res = solver->solve();
    if (!res) { status[i] = 5; continue; }
    status[i] = 0;
    out4[4 * i + 0] = res->value();
    out4[4 * i + 1] = res->delta();
    out4[4 * i + 2] = res->gamma();
    out4[4 * i + 3] = res->theta();
    if (out_dims) {
      out_dims[2 * i + 0] = static_cast<int64_t>(res->grid()->n_space());
      out_dims[2 * i + 1] = static_cast<int64_t>(res->grid()->time().n_steps());
    }
  }
  return 0;
}

// Explicit PDEGridConfig per option: kind 2 = GridSpec::sinh_spaced(x_min,
// x_max, n, alpha), kind 3 = GridSpec::uniform(x_min, x_max, n); nt steps.
int32_t ref_price_explicit(int64_t n, const double* S, const double* K, const double* T,
                           const double* sigma, const double* r, const double* q,
                           const int32_t* is_put, const int32_t* kind, const double* x_min,
                           const double* x_max, const int64_t* nx, const double* alpha,
                           const int64_t* nt, int32_t rannacher, double* out4, int32_t* status) {
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    auto p = make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]);
    auto spec = kind[i] == 3
                    ? GridSpec<double>::uniform(x_min[i], x_max[i], static_cast<size_t>(nx[i]))
                    : GridSpec<double>::sinh_spaced(x_min[i], x_max[i],
                                                    static_cast<size_t>(nx[i]), alpha[i]);
    if (!spec) { status[i] = 1; continue; }
    std::optional<PDEGridSpec> grid = PDEGridSpec{PDEGridConfig{*spec, static_cast<size_t>(nt[i]), {}}};
    auto solver = AmericanOptionSolver::create(p, grid);
    if (!solver) { status[i] = 1; continue; }
    TRBDF2Config cfg;
    cfg.rannacher_startup = rannacher != 0;
    solver->set_trbdf2_config(cfg);
    auto res = solver->solve();
    if (!res) { status[i] = 5; continue; }
    status[i] = 0;
    out4[4 * i + 0] = res->value();
    out4[4 * i + 1] = res->delta();
    out4[4 * i + 2] = res->gamma();
    out4[4 * i + 3] = res->theta();
  }
  return 0;
}

// One option: return the spatial grid and the final / previous solution
// vectors (normalised V/K), for element-wise comparisons.
int32_t ref_price_solution(double S, double K, double T, double sigma, double r,
                           double q, int32_t is_put, int64_t nx, int64_t nt,
                           int64_t cap, double* x_out, double* u_out,
                           double* uprev_out, int64_t* n_out) {
  auto p = make_params(S, K, T, sigma, r, q, is_put);
  auto grid = grid_for(p, nx, nt, 0.0);
  auto solver = AmericanOptionSolver::create(p, grid);
  if (!solver) return 1;
  auto res = solver->solve();
  if (!res) return 5;
  auto g = res->grid();
  const int64_t m = static_cast<int64_t>(g->n_space());
  *n_out = m;
  if (m > cap) return 2;
  auto x = g->x();
  auto u = g->solution();
  auto up = g->solution_prev();
  for (int64_t i = 0; i < m; ++i) { x_out[i] = x[i]; u_out[i] = u[i]; uprev_out[i] = up[i]; }
  return 0;
}

// Prices on a frozen grid: the spatial GridSpec comes from the grid rule
// (estimate_pde_grid pinned to nx points) for the base option (gS, gK, gT,
// gsigma), then every option i is solved on PDEGridConfig{that spec, nt[i]}
// with its own parameters.  Central differences of these prices are the
// reference's frozen-grid sensitivities (the auto grid moves with the
// volatility and the strike, so differences through it jump).
int32_t ref_price_frozen(int64_t n, const double* S, const double* K, const double* T,
                         const double* sigma, const double* r, const double* q,
                         const int32_t* is_put, const double* gS, const double* gK,
                         const double* gT, const double* gsigma, const int64_t* nx,
                         const int64_t* nt, int32_t n_threads, double* out4, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 4)
  for (int64_t i = 0; i < n; ++i) {
    auto pg = make_params(gS[i], gK[i], gT[i], gsigma[i], r[i], q[i], is_put[i]);
    GridAccuracyParams acc;
    acc.min_spatial_points = static_cast<size_t>(nx[i]);
    acc.max_spatial_points = static_cast<size_t>(nx[i]);
    auto [spec, td] = estimate_pde_grid(pg, acc);
    (void)td;
    std::optional<PDEGridSpec> grid = PDEGridSpec{PDEGridConfig{spec, static_cast<size_t>(nt[i]), {}}};
    auto p = make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]);
    auto solver = AmericanOptionSolver::create(p, grid);
    if (!solver) { status[i] = 1; continue; }
    auto res = solver->solve();
    if (!res) { status[i] = 5; continue; }
    status[i] = 0;
    out4[4 * i + 0] = res->value();
    out4[4 * i + 1] = res->delta();
    out4[4 * i + 2] = res->gamma();
    out4[4 * i + 3] = res->theta();
  }
  return 0;
}

// Grid only (estimate_pde_grid + GridSpec::generate), for the host grid code.
int32_t ref_make_grid(double S, double K, double T, double sigma, int64_t nx,
                      int64_t cap, double* x_out, int64_t* n_out, int64_t* nt_out) {
  auto p = make_params(S, K, T, sigma, 0.05, 0.0, 1);
  std::pair<GridSpec<double>, TimeDomain> g = [&] {
    if (nx <= 0) return estimate_pde_grid(p);
    GridAccuracyParams acc;
    acc.min_spatial_points = static_cast<size_t>(nx);
    acc.max_spatial_points = static_cast<size_t>(nx);
    return estimate_pde_grid(p, acc);
  }();
  auto buf = g.first.generate();
  *n_out = static_cast<int64_t>(buf.size());
  *nt_out = static_cast<int64_t>(g.second.n_steps());
  if (*n_out > cap) return 2;
  for (size_t i = 0; i < buf.size(); ++i) x_out[i] = buf[i];
  return 0;
}

// FDM implied volatility through IVSolver::solve (Brent,
// src/option/iv_solver.cpp:133-242).  Each quote gets its own PDEGridConfig
// built by the grid rule at grid_sigma[i] (the vol its price was made with),
// so the objective is smooth in sigma.  out3 = [iv, iterations, final_error].
int32_t ref_iv_batch(int64_t n, const double* S, const double* K, const double* T,
                     const double* r, const double* q, const int32_t* is_put,
                     const double* price, const double* grid_sigma,
                     const int64_t* nx, const int64_t* nt, int32_t n_threads,
                     double* out3, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    IVQuery query;
    query.spot = S[i];
    query.strike = K[i];
    query.maturity = T[i];
    query.rate = r[i];
    query.dividend_yield = q[i];
    query.option_type = is_put[i] ? OptionType::PUT : OptionType::CALL;
    query.market_price = price[i];
    IVSolverConfig cfg;
    if (nx && nx[i] > 0) {
      auto p = make_params(S[i], K[i], T[i], grid_sigma[i], r[i], q[i], is_put[i]);
      cfg.grid = *grid_for(p, nx[i], nt[i], 0.0);
    }
    IVSolver solver(cfg);
    auto res = solver.solve(query);
    if (!res) {
      status[i] = 10 + static_cast<int32_t>(res.error().code);
      out3[3 * i + 0] = NAN;
      out3[3 * i + 1] = static_cast<double>(res.error().iterations);
      out3[3 * i + 2] = res.error().final_error;
      continue;
    }
    status[i] = 0;
    out3[3 * i + 0] = res->implied_vol;
    out3[3 * i + 1] = static_cast<double>(res->iterations);
    out3[3 * i + 2] = res->final_error;
  }
  return 0;
}

// 4D cubic B-spline: knots from clamped_knots_cubic (bspline_basis.hpp:47-91)
// on each axis grid, then BSplineND<double,4>::eval (bspline_nd.hpp:133-157).
// sizes[4]; grids concatenated; coeffs row-major [d0][d1][d2][d3]; q n x 4.
int32_t ref_bspline4d_eval(const int64_t* sizes, const double* grids, const double* coeffs,
                           const double* q, int64_t n, double* out, double* knots_out) {
  std::array<std::vector<double>, 4> g, k;
  size_t off = 0, total = 1, koff = 0;
  for (int d = 0; d < 4; ++d) {
    g[d].assign(grids + off, grids + off + sizes[d]);
    off += static_cast<size_t>(sizes[d]);
    k[d] = clamped_knots_cubic(g[d]);
    total *= static_cast<size_t>(sizes[d]);
    if (knots_out) {
      for (size_t j = 0; j < k[d].size(); ++j) knots_out[koff + j] = k[d][j];
      koff += k[d].size();
    }
  }
  std::vector<double> c(coeffs, coeffs + total);
  auto sp = BSplineND<double, 4>::create(g, k, std::move(c));
  if (!sp) return 1;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    out[i] = sp->eval({q[4 * i + 0], q[4 * i + 1], q[4 * i + 2], q[4 * i + 3]});
  return 0;
}

// Separable 4D collocation fit (BSplineNDSeparable<double,4>::create + fit,
// src/math/bspline/bspline_nd_separable.hpp:127-230), with its LAPACKE calls
// forwarded by lapacke_stubs.c.  values row-major [d0][d1][d2][d3] ->
// coeffs; residual4 / cond4: the per-axis diagnostics.  Returns 0, or 1
// when create or fit fails.
int32_t ref_bspline4d_fit(const int64_t* sizes, const double* grids, const double* values,
                          double tolerance, double* coeffs, double* residual4, double* cond4) {
  std::array<std::vector<double>, 4> g;
  size_t off = 0, total = 1;
  for (int d = 0; d < 4; ++d) {
    g[d].assign(grids + off, grids + off + sizes[d]);
    off += static_cast<size_t>(sizes[d]);
    total *= static_cast<size_t>(sizes[d]);
  }
  auto fitter = BSplineNDSeparable<double, 4>::create(g);
  if (!fitter) return 1;
  BSplineNDSeparableConfig<double> cfg;
  cfg.tolerance = tolerance;
  auto res = fitter->fit(std::vector<double>(values, values + total), cfg);
  if (!res) return 1;
  for (size_t i = 0; i < total; ++i) coeffs[i] = res->coefficients[i];
  for (int d = 0; d < 4; ++d) {
    residual4[d] = res->max_residual_per_axis[d];
    cond4[d] = res->condition_per_axis[d];
  }
  return 0;
}

// Price-table PDE sweep + extraction (PriceTableBuilderND<4>::make_batch,
// solve_batch, extract_tensor; src/option/table/bspline/bspline_builder.cpp:
// 198-480).  grid_kind 0: GridAccuracyParams{}; 1: PDEGridConfig with
// GridSpec::sinh_spaced(x_min, x_max, nx, alpha) and n_time steps.
// out: tensor [m][tau][sigma][r]; dims: per (sigma, r) slice {n_space, n_time}.
int32_t ref_table_sweep(const double* m, int64_t nm, const double* tau, int64_t ntau,
                        const double* sig, int64_t ns, const double* rr, int64_t nr,
                        double K_ref, double q, int32_t is_put, int32_t grid_kind,
                        double x_min, double x_max, int64_t nx, double alpha, int64_t n_time,
                        double* out, int64_t* dims) {
  PriceTableConfig cfg;
  cfg.option_type = is_put ? OptionType::PUT : OptionType::CALL;
  cfg.K_ref = K_ref;
  cfg.dividends.dividend_yield = q;
  if (grid_kind == 1) {
    auto spec = GridSpec<double>::sinh_spaced(x_min, x_max, static_cast<size_t>(nx), alpha);
    if (!spec) return 1;
    cfg.pde_grid = PDEGridConfig{*spec, static_cast<size_t>(n_time), {}};
  }
  PriceTableBuilderND<4> b(cfg);
  PriceTableAxesND<4> axes;
  axes.grids[0].assign(m, m + nm);
  axes.grids[1].assign(tau, tau + ntau);
  axes.grids[2].assign(sig, sig + ns);
  axes.grids[3].assign(rr, rr + nr);
  auto batch = b.make_batch(axes);
  auto res = testing::PriceTableBuilderAccess<4>::solve_batch(b, batch, axes);
  for (size_t i = 0; i < res.results.size(); ++i) {
    if (res.results[i]) {
      dims[2 * i] = static_cast<int64_t>(res.results[i]->grid()->n_space());
      dims[2 * i + 1] = static_cast<int64_t>(res.results[i]->grid()->time().n_steps());
    } else {
      dims[2 * i] = dims[2 * i + 1] = -1;
    }
  }
  auto ext = b.extract_tensor(res, axes);
  if (!ext) return 2;
  for (int64_t i = 0; i < nm; ++i)
    for (int64_t j = 0; j < ntau; ++j)
      for (int64_t k = 0; k < ns; ++k)
        for (int64_t l = 0; l < nr; ++l)
          out[((i * ntau + j) * ns + k) * nr + l] = ext->tensor.view[i, j, k, l];
  return 0;
}

// Standard price table over given spline coefficients
// (make_bspline_surface, src/option/table/bspline/bspline_surface.cpp:9-37)
// and its price(spot, strike, tau, sigma, rate) (EEPLayer over TransformLeaf).
// p: n x 5 records {spot, strike, tau, sigma, rate}.
int32_t ref_surface_price(const int64_t* sizes, const double* grids, const double* coeffs,
                          double K_ref, double q, int32_t is_put, const double* p, int64_t n,
                          double* out) {
  std::array<std::vector<double>, 4> g, k;
  size_t off = 0, total = 1;
  for (int d = 0; d < 4; ++d) {
    g[d].assign(grids + off, grids + off + sizes[d]);
    off += static_cast<size_t>(sizes[d]);
    k[d] = clamped_knots_cubic(g[d]);
    total *= static_cast<size_t>(sizes[d]);
  }
  std::vector<double> c(coeffs, coeffs + total);
  auto sp = BSplineND<double, 4>::create(g, k, std::move(c));
  if (!sp) return 1;
  auto shared = std::make_shared<const BSplineND<double, 4>>(std::move(sp.value()));
  auto table = make_bspline_surface(shared, K_ref, q, is_put ? OptionType::PUT : OptionType::CALL);
  if (!table) return 2;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i)
    out[i] = table->price(p[5 * i], p[5 * i + 1], p[5 * i + 2], p[5 * i + 3], p[5 * i + 4]);
  return 0;
}

// eep_decompose over BSplineTensorAccessor with AnalyticalEEP
// (src/option/table/eep/eep_decomposer.hpp:60-80): tensor [m][tau][sigma][r]
// of V/K_ref in, EEP out, in place.
int32_t ref_eep_decompose(const double* m, int64_t nm, const double* tau, int64_t ntau,
                          const double* sig, int64_t ns, const double* rr, int64_t nr,
                          double K_ref, double q, int32_t is_put, double* tensor) {
  PriceTableAxesND<4> axes;
  axes.grids[0].assign(m, m + nm);
  axes.grids[1].assign(tau, tau + ntau);
  axes.grids[2].assign(sig, sig + ns);
  axes.grids[3].assign(rr, rr + nr);
  auto t = PriceTensorND<4>::create({static_cast<size_t>(nm), static_cast<size_t>(ntau),
                                     static_cast<size_t>(ns), static_cast<size_t>(nr)});
  if (!t) return 1;
  for (int64_t i = 0; i < nm; ++i)
    for (int64_t j = 0; j < ntau; ++j)
      for (int64_t a = 0; a < ns; ++a)
        for (int64_t l = 0; l < nr; ++l)
          t->view[i, j, a, l] = tensor[((i * ntau + j) * ns + a) * nr + l];
  BSplineTensorAccessor acc(*t, axes, K_ref);
  eep_decompose(acc, AnalyticalEEP(is_put ? OptionType::PUT : OptionType::CALL, q));
  for (int64_t i = 0; i < nm; ++i)
    for (int64_t j = 0; j < ntau; ++j)
      for (int64_t a = 0; a < ns; ++a)
        for (int64_t l = 0; l < nr; ++l)
          tensor[((i * ntau + j) * ns + a) * nr + l] = t->view[i, j, a, l];
  return 0;
}

// The standard table's vega (EEPLayer::vega over TransformLeaf::vega);
// p as for ref_surface_price.
int32_t ref_surface_vega(const int64_t* sizes, const double* grids, const double* coeffs,
                         double K_ref, double q, int32_t is_put, const double* p, int64_t n,
                         double* out) {
  std::array<std::vector<double>, 4> g, k;
  size_t off = 0, total = 1;
  for (int d = 0; d < 4; ++d) {
    g[d].assign(grids + off, grids + off + sizes[d]);
    off += static_cast<size_t>(sizes[d]);
    k[d] = clamped_knots_cubic(g[d]);
    total *= static_cast<size_t>(sizes[d]);
  }
  std::vector<double> c(coeffs, coeffs + total);
  auto sp = BSplineND<double, 4>::create(g, k, std::move(c));
  if (!sp) return 1;
  auto shared = std::make_shared<const BSplineND<double, 4>>(std::move(sp.value()));
  auto table = make_bspline_surface(shared, K_ref, q, is_put ? OptionType::PUT : OptionType::CALL);
  if (!table) return 2;
  for (int64_t i = 0; i < n; ++i)
    out[i] = table->vega(p[5 * i], p[5 * i + 1], p[5 * i + 2], p[5 * i + 3], p[5 * i + 4]);
  return 0;
}

// InterpolatedIVSolver<BSplinePriceTable>::solve_batch on the standard table.
// cfg = {max_iter, tolerance, sigma_min, sigma_max, vega_threshold};
// queries n x 7 {spot, strike, tau, rate, q, is_put, price}; out n x 3
// {iv, iterations, final_error}; status = the C ABI's map_iv_error
// (src/ffi/mango_c_api.cpp:124-141) of each result (0 on success).
int32_t ref_surface_iv(const int64_t* sizes, const double* grids, const double* coeffs,
                       double K_ref, double q, int32_t is_put, const double* cfg,
                       const double* qs, int64_t n, double* out, int32_t* status) {
  std::array<std::vector<double>, 4> g, k;
  size_t off = 0, total = 1;
  for (int d = 0; d < 4; ++d) {
    g[d].assign(grids + off, grids + off + sizes[d]);
    off += static_cast<size_t>(sizes[d]);
    k[d] = clamped_knots_cubic(g[d]);
    total *= static_cast<size_t>(sizes[d]);
  }
  std::vector<double> c(coeffs, coeffs + total);
  auto sp = BSplineND<double, 4>::create(g, k, std::move(c));
  if (!sp) return 1;
  auto shared = std::make_shared<const BSplineND<double, 4>>(std::move(sp.value()));
  auto table = make_bspline_surface(shared, K_ref, q, is_put ? OptionType::PUT : OptionType::CALL);
  if (!table) return 2;
  InterpolatedIVSolverConfig sc;
  sc.max_iter = static_cast<size_t>(cfg[0]);
  sc.tolerance = cfg[1];
  sc.sigma_min = cfg[2];
  sc.sigma_max = cfg[3];
  sc.vega_threshold = cfg[4];
  auto solver = InterpolatedIVSolver<BSplinePriceTable>::create(std::move(*table), sc);
  if (!solver) return 3;
  std::vector<IVQuery> queries;
  for (int64_t i = 0; i < n; ++i) {
    const double* r = qs + 7 * i;
    OptionSpec spec{.spot = r[0], .strike = r[1], .maturity = r[2], .rate = r[3],
                    .dividend_yield = r[4], .option_type = r[5] != 0.0 ? OptionType::PUT : OptionType::CALL};
    queries.emplace_back(spec, r[6]);
  }
  auto res = solver->solve_batch(queries);
  for (int64_t i = 0; i < n; ++i) {
    const auto& r = res.results[i];
    if (r) {
      out[3 * i] = r->implied_vol;
      out[3 * i + 1] = static_cast<double>(r->iterations);
      out[3 * i + 2] = r->final_error;
      status[i] = 0;
    } else {
      out[3 * i] = NAN;
      out[3 * i + 1] = static_cast<double>(r.error().iterations);
      out[3 * i + 2] = r.error().final_error;
      switch (r.error().code) {
        case IVErrorCode::ArbitrageViolation: status[i] = 2; break;
        case IVErrorCode::BracketingFailed: status[i] = 4; break;
        case IVErrorCode::MaxIterationsExceeded: status[i] = 3; break;
        case IVErrorCode::NegativeSpot:
        case IVErrorCode::NegativeStrike:
        case IVErrorCode::NegativeMaturity:
        case IVErrorCode::NegativeMarketPrice:
        case IVErrorCode::InvalidGridConfig:
        case IVErrorCode::OptionTypeMismatch:
        case IVErrorCode::DividendYieldMismatch: status[i] = 1; break;
        default: status[i] = 5; break;
      }
    }
  }
  return 0;
}


// BatchAmericanOptionSolver::solve_batch with use_shared_grid = true
// (src/option/american_option_batch.cpp:272-302): the normalized chain when
// use_normalized and the batch is eligible, else the regular shared-grid
// batch.  kind 0 = no custom grid; 2 / 3 = PDEGridConfig{sinh_spaced /
// uniform(x_min, x_max, nx[, alpha]), nt}; 1 = GridAccuracyParams with
// min == max == nx.  out_dims = [n_space, n_time] per option.
int32_t ref_batch_shared(int64_t n, const double* S, const double* K, const double* T,
                         const double* sigma, const double* r, const double* q,
                         const int32_t* is_put, int32_t use_normalized, int32_t kind,
                         double x_min, double x_max, int64_t nx, double alpha, int64_t nt,
                         int32_t n_threads, double* out4, int64_t* out_dims, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  std::vector<PricingParams> ps;
  ps.reserve(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) ps.push_back(make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]));
  std::optional<PDEGridSpec> custom;
  if (kind == 2 || kind == 3) {
    auto spec = kind == 3 ? GridSpec<double>::uniform(x_min, x_max, static_cast<size_t>(nx))
                          : GridSpec<double>::sinh_spaced(x_min, x_max, static_cast<size_t>(nx), alpha);
    if (!spec) return 1;
    custom = PDEGridSpec{PDEGridConfig{*spec, static_cast<size_t>(nt), {}}};
  } else if (kind == 1) {
    GridAccuracyParams acc;
    acc.min_spatial_points = static_cast<size_t>(nx);
    acc.max_spatial_points = static_cast<size_t>(nx);
    custom = PDEGridSpec{acc};
  }
  BatchAmericanOptionSolver solver;
  solver.set_use_normalized(use_normalized != 0);
  auto res = solver.solve_batch(ps, true, nullptr, custom);
  for (int64_t i = 0; i < n; ++i) {
    const auto& ri = res.results[static_cast<size_t>(i)];
    if (!ri) { status[i] = 5; continue; }
    status[i] = 0;
    out4[4 * i + 0] = ri->value();
    out4[4 * i + 1] = ri->delta();
    out4[4 * i + 2] = ri->gamma();
    out4[4 * i + 3] = ri->theta();
    out_dims[2 * i + 0] = static_cast<int64_t>(ri->grid()->n_space());
    out_dims[2 * i + 1] = static_cast<int64_t>(ri->grid()->time().n_steps());
  }
  return 0;
}


// Options with a yield curve and/or discrete dividends through the
// reference's AmericanOptionSolver.  Per option i: curve points
// [curve_off[i], curve_off[i] + curve_n[i]) (none: constant rate r[i]),
// dividends [div_off[i], div_off[i] + div_n[i]).  kind 0 = the solver's own
// grid (AmericanOptionSolver::create(p), as mango_price_american);
// 1 = estimate_pde_grid with min == max == nx[i], then PDEGridConfig{spec,
// nt[i], dividend times} (nt[i] == 0: the estimate's own time domain);
// 2 / 3 = PDEGridConfig{sinh_spaced / uniform, nt[i], dividend times}.  The
// dividend times are the taus in (0, T), as solve_regular_batch attaches
// them.
int32_t ref_price_tv(int64_t n, const double* S, const double* K, const double* T,
                     const double* sigma, const double* r, const double* q, const int32_t* is_put,
                     const int64_t* curve_off, const int64_t* curve_n, const double* curve_t,
                     const double* curve_ld, const int64_t* div_off, const int64_t* div_n,
                     const double* div_t, const double* div_amt, const int32_t* kind,
                     const int64_t* nx, const int64_t* nt, const double* x_min, const double* x_max,
                     const double* alpha, int32_t rannacher, int32_t n_threads, double* out4,
                     int64_t* out_dims, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    auto p = make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]);
    if (curve_n[i] > 0) {
      std::vector<TenorPoint> pts;
      for (int64_t j = 0; j < curve_n[i]; ++j)
        pts.push_back(TenorPoint{curve_t[curve_off[i] + j], curve_ld[curve_off[i] + j]});
      auto c = YieldCurve::from_points(std::move(pts));
      if (!c) { status[i] = 1; continue; }
      p.rate = *c;
    }
    std::vector<double> taus;
    for (int64_t j = 0; j < div_n[i]; ++j) {
      p.discrete_dividends.push_back(Dividend{div_t[div_off[i] + j], div_amt[div_off[i] + j]});
      const double tau = p.maturity - div_t[div_off[i] + j];
      if (tau > 0.0 && tau < p.maturity) taus.push_back(tau);
    }
    std::optional<PDEGridSpec> grid;
    if (kind[i] == 1) {
      GridAccuracyParams acc;
      acc.min_spatial_points = static_cast<size_t>(nx[i]);
      acc.max_spatial_points = static_cast<size_t>(nx[i]);
      if (nt[i] == 0) {
        grid = PDEGridSpec{acc};
      } else {
        auto [spec, td] = estimate_pde_grid(p, acc);
        (void)td;
        grid = PDEGridSpec{PDEGridConfig{spec, static_cast<size_t>(nt[i]), taus}};
      }
    } else if (kind[i] == 2 || kind[i] == 3) {
      auto spec = kind[i] == 3 ? GridSpec<double>::uniform(x_min[i], x_max[i], static_cast<size_t>(nx[i]))
                               : GridSpec<double>::sinh_spaced(x_min[i], x_max[i],
                                                               static_cast<size_t>(nx[i]), alpha[i]);
      if (!spec) { status[i] = 1; continue; }
      grid = PDEGridSpec{PDEGridConfig{*spec, static_cast<size_t>(nt[i]), taus}};
    }
    auto solver = AmericanOptionSolver::create(p, grid);
    if (!solver) { status[i] = 1; continue; }
    TRBDF2Config cfg;
    cfg.rannacher_startup = rannacher != 0;
    solver->set_trbdf2_config(cfg);
    auto res = solver->solve();
    if (!res) { status[i] = 5; continue; }
    status[i] = 0;
    out4[4 * i + 0] = res->value();
    out4[4 * i + 1] = res->delta();
    out4[4 * i + 2] = res->gamma();
    out4[4 * i + 3] = res->theta();
    out_dims[2 * i + 0] = static_cast<int64_t>(res->grid()->n_space());
    out_dims[2 * i + 1] = static_cast<int64_t>(res->grid()->time().n_steps());
  }
  return 0;
}


// ref_batch_shared for options with yield curves and dividends (the
// schedules as in ref_price_tv).
int32_t ref_batch_shared_tv(int64_t n, const double* S, const double* K, const double* T,
                            const double* sigma, const double* r, const double* q,
                            const int32_t* is_put, const int64_t* curve_off, const int64_t* curve_n,
                            const double* curve_t, const double* curve_ld, const int64_t* div_off,
                            const int64_t* div_n, const double* div_t, const double* div_amt,
                            int32_t use_normalized, int32_t kind, double x_min, double x_max,
                            int64_t nx, double alpha, int64_t nt, int32_t n_threads, double* out4,
                            int64_t* out_dims, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
  std::vector<PricingParams> ps;
  for (int64_t i = 0; i < n; ++i) {
    auto p = make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]);
    if (curve_n[i] > 0) {
      std::vector<TenorPoint> pts;
      for (int64_t j = 0; j < curve_n[i]; ++j)
        pts.push_back(TenorPoint{curve_t[curve_off[i] + j], curve_ld[curve_off[i] + j]});
      auto c = YieldCurve::from_points(std::move(pts));
      if (!c) return 1;
      p.rate = *c;
    }
    for (int64_t j = 0; j < div_n[i]; ++j)
      p.discrete_dividends.push_back(Dividend{div_t[div_off[i] + j], div_amt[div_off[i] + j]});
    ps.push_back(std::move(p));
  }
  std::optional<PDEGridSpec> custom;
  if (kind == 2 || kind == 3) {
    auto spec = kind == 3 ? GridSpec<double>::uniform(x_min, x_max, static_cast<size_t>(nx))
                          : GridSpec<double>::sinh_spaced(x_min, x_max, static_cast<size_t>(nx), alpha);
    if (!spec) return 1;
    custom = PDEGridSpec{PDEGridConfig{*spec, static_cast<size_t>(nt), {}}};
  } else if (kind == 1) {
    GridAccuracyParams acc;
    acc.min_spatial_points = static_cast<size_t>(nx);
    acc.max_spatial_points = static_cast<size_t>(nx);
    custom = PDEGridSpec{acc};
  }
  BatchAmericanOptionSolver solver;
  solver.set_use_normalized(use_normalized != 0);
  auto res = solver.solve_batch(ps, true, nullptr, custom);
  for (int64_t i = 0; i < n; ++i) {
    const auto& ri = res.results[static_cast<size_t>(i)];
    if (!ri) { status[i] = 5; continue; }
    status[i] = 0;
    out4[4 * i + 0] = ri->value();
    out4[4 * i + 1] = ri->delta();
    out4[4 * i + 2] = ri->gamma();
    out4[4 * i + 3] = ri->theta();
    out_dims[2 * i + 0] = static_cast<int64_t>(ri->grid()->n_space());
    out_dims[2 * i + 1] = static_cast<int64_t>(ri->grid()->time().n_steps());
  }
  return 0;
}


// CRC64::update of the reference (src/support/crc64.cpp).
uint64_t ref_crc64_update(uint64_t crc, const uint8_t* data, uint64_t n) {
  return CRC64::update(crc, data, static_cast<size_t>(n));
}


// IVSolver::solve for quotes with yield curves and/or discrete dividends
// (schedules as in ref_price_tv).  The grid: estimate_pde_grid of the quote
// at grid_sigma with min == max == nx (dividends included, so the lower
// bound is widened as for the option), as PDEGridConfig{spec, nt}; the
// solver adds the dividend times (iv_solver.cpp:82-96).
int32_t ref_iv_batch_tv(int64_t n, const double* S, const double* K, const double* T,
                        const double* r, const double* q, const int32_t* is_put,
                        const double* price, const double* grid_sigma, const int64_t* nx,
                        const int64_t* nt, const int64_t* curve_off, const int64_t* curve_n,
                        const double* curve_t, const double* curve_ld, const int64_t* div_off,
                        const int64_t* div_n, const double* div_t, const double* div_amt,
                        int32_t n_threads, double* out3, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    IVQuery query;
    query.spot = S[i];
    query.strike = K[i];
    query.maturity = T[i];
    query.rate = r[i];
    query.dividend_yield = q[i];
    query.option_type = is_put[i] ? OptionType::PUT : OptionType::CALL;
    query.market_price = price[i];
    auto p = make_params(S[i], K[i], T[i], grid_sigma[i], r[i], q[i], is_put[i]);
    if (curve_n[i] > 0) {
      std::vector<TenorPoint> pts;
      for (int64_t j = 0; j < curve_n[i]; ++j)
        pts.push_back(TenorPoint{curve_t[curve_off[i] + j], curve_ld[curve_off[i] + j]});
      auto c = YieldCurve::from_points(std::move(pts));
      if (!c) { status[i] = 1; continue; }
      query.rate = *c;
      p.rate = *c;
    }
    for (int64_t j = 0; j < div_n[i]; ++j) {
      const Dividend d{div_t[div_off[i] + j], div_amt[div_off[i] + j]};
      query.discrete_dividends.push_back(d);
      p.discrete_dividends.push_back(d);
    }
    GridAccuracyParams acc;
    acc.min_spatial_points = static_cast<size_t>(nx[i]);
    acc.max_spatial_points = static_cast<size_t>(nx[i]);
    auto [spec, td] = estimate_pde_grid(p, acc);
    (void)td;
    IVSolverConfig cfg;
    cfg.grid = PDEGridConfig{spec, static_cast<size_t>(nt[i]), {}};
    IVSolver solver(cfg);
    auto res = solver.solve(query);
    if (!res) {
      status[i] = 10 + static_cast<int32_t>(res.error().code);
      out3[3 * i + 0] = NAN;
      out3[3 * i + 1] = static_cast<double>(res.error().iterations);
      out3[3 * i + 2] = res.error().final_error;
      continue;
    }
    status[i] = 0;
    out3[3 * i + 0] = res->implied_vol;
    out3[3 * i + 1] = static_cast<double>(res->iterations);
    out3[3 * i + 2] = res->final_error;
  }
  return 0;
}


// AmericanOptionResult::value_at (american_option_result.cpp:29-45) at
// spot2[i] for options priced on the fixed-size grid rule (nx, nt).
int32_t ref_value_at(int64_t n, const double* S, const double* K, const double* T,
                     const double* sigma, const double* r, const double* q, const int32_t* is_put,
                     const int64_t* nx, const int64_t* nt, const double* spot2, int32_t n_threads,
                     double* out, int32_t* status) {
  if (n_threads > 0) omp_set_num_threads(n_threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t i = 0; i < n; ++i) {
    auto p = make_params(S[i], K[i], T[i], sigma[i], r[i], q[i], is_put[i]);
    auto grid = grid_for(p, nx[i], nt[i], 0.0);
    auto solver = AmericanOptionSolver::create(p, grid);
    if (!solver) { status[i] = 1; continue; }
    auto res = solver->solve();
    if (!res) { status[i] = 5; continue; }
    status[i] = 0;
    out[i] = res->value_at(spot2[i]);
  }
  return 0;
}


// The standard table's delta, gamma, theta and rho (PriceTable over
// EEPLayer<TransformLeaf>: eep_layer.hpp:33-76, transform_leaf.hpp:46-90),
// p n x 5 {spot, strike, tau, sigma, rate}; out n x 4; status 0 or 1 + the
// GreekError code.
int32_t ref_surface_greeks(const int64_t* sizes, const double* grids, const double* coeffs,
                           double K_ref, double q, int32_t is_put, const double* p, int64_t n,
                           double* out, int32_t* status) {
  std::array<std::vector<double>, 4> g, k;
  size_t off = 0, total = 1;
  for (int d = 0; d < 4; ++d) {
    g[d].assign(grids + off, grids + off + sizes[d]);
    off += static_cast<size_t>(sizes[d]);
    k[d] = clamped_knots_cubic(g[d]);
    total *= static_cast<size_t>(sizes[d]);
  }
  std::vector<double> c(coeffs, coeffs + total);
  auto sp = BSplineND<double, 4>::create(g, k, std::move(c));
  if (!sp) return 1;
  auto shared = std::make_shared<const BSplineND<double, 4>>(std::move(sp.value()));
  auto table = make_bspline_surface(shared, K_ref, q, is_put ? OptionType::PUT : OptionType::CALL);
  if (!table) return 2;
  for (int64_t i = 0; i < n; ++i) {
    PricingParams pp = make_params(p[5 * i], p[5 * i + 1], p[5 * i + 2], p[5 * i + 3], p[5 * i + 4], q, is_put);
    auto d = table->delta(pp);
    auto ga = table->gamma(pp);
    auto th = table->theta(pp);
    auto rh = table->rho(pp);
    if (!d || !ga || !th || !rh) { status[i] = 1; continue; }
    status[i] = 0;
    out[4 * i + 0] = *d;
    out[4 * i + 1] = *ga;
    out[4 * i + 2] = *th;
    out[4 * i + 3] = *rh;
  }
  return 0;
}

}  // extern "C"
