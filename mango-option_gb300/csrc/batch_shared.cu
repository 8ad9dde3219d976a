// batch_shared.cu -- BatchAmericanOptionSolver::solve_batch with a shared grid.
//
// Restates the shared-grid routes of BatchAmericanOptionSolver::solve_batch
// (src/option/american_option_batch.cpp:272-302):
//   is_normalized_eligible (american_option_batch.cpp:26-107): one option
//     type, no discrete dividends, positive spot and strike, and the grid of
//     the first option (estimate_pde_grid) within the width / spacing limits
//     with margins around the batch's log-moneyness range;
//   solve_normalized_chain (american_option_batch.cpp:313-382): options
//     grouped by (sigma, r, q, maturity, type) (group_by_pde_parameters,
//     american_option_batch.cpp:219-268, tolerance 1e-10, first match), one
//     S = K = 1 solve per group on the shared grid of that single option
//     (estimate_batch_pde_grid, or the custom grid), every option's
//     AmericanOptionResult read from its group's solution with its own spot
//     and strike;
//   solve_regular_batch with use_shared_grid (american_option_batch.cpp:
//     384-518): one grid for the whole batch (estimate_batch_pde_grid,
//     src/option/grid_spec_types.cpp:120-177, or the custom grid resolved for
//     the first option), each option marched on it with its own maturity and
//     the shared step count.
// The marches are ordinary device batches; the chain's per-option
// functionals run in chain_outputs_kernel (march.cu).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine.hpp"

namespace mgpu {

namespace {

// BatchAmericanOptionSolver limits (src/option/american_option_batch.hpp:219-221).
constexpr double kMaxWidth = 5.8;
constexpr double kMaxDx = 0.05;
constexpr double kMinMarginAbs = 0.35;

// estimate_batch_pde_grid: the union of the options' estimated x ranges
// (each widened for its dividends), their largest n_space, and the batch
// time domain over the longest maturity: from_n_steps at the largest step
// count, or, when any option has a dividend inside (0, T_max),
// with_mandatory_points at that step (capped) through the union of the
// dividend times.  *nt is that domain's step count.
void estimate_batch_grid(const std::vector<const MangoPricingParams*>& ps, const Accuracy& acc,
                         GridSpec* spec, int64_t* nt) {
  double gmin = 1e300, gmax = -1e300;
  int64_t gnx = 0, gnt = 0;
  std::vector<double> scratch, taus, tp;
  for (const MangoPricingParams* p : ps) {
    GridSpec s;
    int64_t n_t = 0;
    taus.clear();
    double max_dk = 0.0;
    for (uint64_t j = 0; j < p->n_dividends; ++j) {
      const double tau = p->maturity - p->dividends[j].calendar_time;
      if (tau > 0.0 && tau < p->maturity) {
        taus.push_back(tau);
        max_dk = std::max(max_dk, p->dividends[j].amount / p->strike);
      }
    }
    estimate_grid_div(p->spot, p->strike, p->maturity, p->volatility, acc, taus, max_dk, &s, &n_t,
                      &tp, &scratch);
    gmin = std::min(gmin, s.x_min);
    gmax = std::max(gmax, s.x_max);
    gnx = std::max<int64_t>(gnx, s.n);
    gnt = std::max<int64_t>(gnt, n_t);
  }
  double t_max = 0.0;
  for (const MangoPricingParams* p : ps) t_max = std::max(t_max, p->maturity);
  std::vector<double> all_tau;
  for (const MangoPricingParams* p : ps)
    for (uint64_t j = 0; j < p->n_dividends; ++j) {
      const double tau = p->maturity - p->dividends[j].calendar_time;
      if (tau > 0.0 && tau < t_max) all_tau.push_back(tau);
    }
  if (!all_tau.empty()) {
    const double global_dt = t_max / static_cast<double>(gnt);
    const double cap = t_max / static_cast<double>(acc.max_steps);
    const double dt_capped = (global_dt < cap) ? cap : global_dt;
    time_points(0.0, t_max, dt_capped, all_tau, &tp, &gnt);
  }
  GridSpec s;
  // multi_sinh_spaced with one cluster at x = 0 (grid.hpp:110-160 checks),
  // else the plain sinh fallback.
  const bool ok = gnx >= 2 && gmin < gmax && 0.0 >= gmin && 0.0 <= gmax && acc.alpha > 0;
  if (ok) {
    s.type = GridSpec::MultiSinh;
    s.n_clusters = 1;
    s.x_min = gmin;
    s.x_max = gmax;
    s.n = gnx;
    s.c_center[0] = 0.0;
    s.c_alpha[0] = acc.alpha;
    s.c_weight[0] = 1.0;
  } else {
    s = sinh_spec(gmin, gmax, gnx, acc.alpha);
  }
  *spec = s;
  *nt = gnt;
}

// Rate comparison of group_by_pde_parameters: constants within 1e-10,
// yield curves equal point by point within 1e-12 (YieldCurve::operator==,
// on the tenor-sorted points).
bool same_rate(const MangoPricingParams& a, const MangoPricingParams& b) {
  if ((a.n_tenor_points == 0) != (b.n_tenor_points == 0)) return false;
  if (a.n_tenor_points == 0) return std::fabs(a.rate_const - b.rate_const) < 1e-10;
  if (a.n_tenor_points != b.n_tenor_points) return false;
  auto sorted = [](const MangoPricingParams& p) {
    std::vector<MangoTenorPoint> v(p.tenor_points, p.tenor_points + p.n_tenor_points);
    std::sort(v.begin(), v.end(),
              [](const MangoTenorPoint& x, const MangoTenorPoint& y) { return x.tenor < y.tenor; });
    return v;
  };
  const auto va = sorted(a), vb = sorted(b);
  for (size_t i = 0; i < va.size(); ++i)
    if (std::fabs(va[i].tenor - vb[i].tenor) > 1e-12 ||
        std::fabs(va[i].log_discount - vb[i].log_discount) > 1e-12)
      return false;
  return true;
}

bool eligible(const MangoPricingParams* params, int64_t n, const Accuracy& acc) {
  if (n <= 0) return false;
  const MangoPricingParams& first = params[0];
  for (int64_t i = 1; i < n; ++i)
    if (params[i].option_type != first.option_type) return false;
  for (int64_t i = 0; i < n; ++i)
    if (params[i].n_dividends != 0) return false;
  for (int64_t i = 0; i < n; ++i)
    if (params[i].spot <= 0.0 || params[i].strike <= 0.0) return false;
  GridSpec s;
  int64_t n_t = 0;
  std::vector<double> scratch;
  estimate_grid(first.spot, first.strike, first.maturity, first.volatility, acc, &s, &n_t, &scratch);
  const double dx = (s.x_max - s.x_min) / static_cast<double>(s.n - 1);
  if (dx > kMaxDx) return false;
  if (s.x_max - s.x_min > kMaxWidth) return false;
  double m_min = 1e300, m_max = -1e300;
  for (int64_t i = 0; i < n; ++i) {
    const double m = params[i].spot / params[i].strike;
    m_min = std::min(m_min, m);
    m_max = std::max(m_max, m);
  }
  const double margin_left = std::log(m_min) - s.x_min;
  const double margin_right = s.x_max - std::log(m_max);
  const double min_margin = std::max(kMinMarginAbs, 6.0 * dx);
  return !(margin_left < min_margin || margin_right < min_margin);
}

}  // namespace
}  // namespace mgpu

using namespace mgpu;

extern "C" MangoStatus mango_gpu_price_american_batch_shared(
    MangoGpuContext* ctx, const MangoPricingParams* params, uint64_t n,
    const MangoGpuGrid* custom_grid, int32_t use_normalized, const MangoGpuTrbdf2* trbdf2,
    MangoGpuAmericanOut* out, uint64_t* out_failed, int32_t* out_route, MangoError* err) {
  if (!ctx || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, params or out");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 26)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^26 options");
    return MANGO_ERR_VALIDATION;
  }
  const int64_t nn = static_cast<int64_t>(n);
  const Accuracy acc = default_accuracy();
  if (n == 0) {
    if (out_failed) *out_failed = 0;
    if (out_route) *out_route = 0;
    return MANGO_OK;
  }
  // A custom grid is resolved for the first option of the solve, as
  // solve_regular_batch's resolve_grid does (american_option_batch.cpp:410-434).
  const bool custom = custom_grid != nullptr;
  std::vector<double> gscratch;
  auto resolve_custom = [&](const MangoPricingParams& p, Resolved* r) {
    return resolve(p, *custom_grid, r, &gscratch);
  };
  MangoGpuBatch* b = nullptr;
  DevBuf d_grp, d_spot, d_strike, d_scratch, d_out;
  auto release = [&]() {
    for (DevBuf* d : {&d_grp, &d_spot, &d_strike, &d_scratch, &d_out}) d->release();
    if (b) destroy_batch(b);
    b = nullptr;
  };
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::vector<std::string> vmsg(static_cast<size_t>(nn));
    std::vector<char> valid(static_cast<size_t>(nn), 0);
    for (int64_t i = 0; i < nn; ++i) {
      vmsg[i] = validate(params[i], true);
      valid[i] = vmsg[i].empty();
    }
    for (int64_t i = 0; i < nn; ++i) {
      std::memset(&out[i], 0, sizeof(out[i]));
      out[i].value = out[i].delta = out[i].gamma = out[i].theta = NAN;
      out[i].status = valid[i] ? MANGO_OK : MANGO_ERR_VALIDATION;
    }
    const bool chain = use_normalized && eligible(params, nn, acc);
    if (out_route) *out_route = chain ? 1 : 0;
    std::string first_err;
    if (chain) {
      // group_by_pde_parameters over the options (first match, 1e-10).
      struct Group {
        double sigma, q, T;
        int32_t type;
        const MangoPricingParams* rep;  // first option: its rate or curve
      };
      std::vector<Group> groups;
      std::vector<int32_t> gof(static_cast<size_t>(nn), -1);
      // The first matching group, found without scanning every group: a
      // group can only match if its volatility lies within 1e-10 of the
      // option's, so groups are indexed by volatility in buckets 1e-10 wide
      // and only the option's bucket and its neighbours (two either side, for
      // the rounding of the bucket index) are tested; the smallest matching
      // group index is the first match in creation order.
      std::unordered_map<int64_t, std::vector<int32_t>> by_sigma;
      auto bucket = [](double v) { return static_cast<int64_t>(std::floor(v / 1e-10)); };
      for (int64_t i = 0; i < nn; ++i) {
        if (!valid[i]) continue;
        const MangoPricingParams& p = params[i];
        int32_t found = -1;
        const int64_t bk = bucket(p.volatility);
        for (int64_t nb = bk - 2; nb <= bk + 2; ++nb) {
          const auto it = by_sigma.find(nb);
          if (it == by_sigma.end()) continue;
          for (const int32_t g : it->second) {
            if (found >= 0 && g >= found) break;  // lists are in creation order
            const Group& G = groups[static_cast<size_t>(g)];
            if (std::fabs(G.sigma - p.volatility) < 1e-10 && same_rate(*G.rep, p) &&
                std::fabs(G.q - p.dividend_yield) < 1e-10 && std::fabs(G.T - p.maturity) < 1e-10 &&
                G.type == p.option_type) {
              found = g;
              break;
            }
          }
        }
        if (found < 0) {
          found = static_cast<int32_t>(groups.size());
          groups.push_back({p.volatility, p.dividend_yield, p.maturity, p.option_type, &p});
          by_sigma[bk].push_back(found);
        }
        gof[i] = found;
      }
      const int64_t ng = static_cast<int64_t>(groups.size());
      std::vector<MangoPricingParams> gp(static_cast<size_t>(ng));
      std::vector<Resolved> res(static_cast<size_t>(ng));
      for (int64_t g = 0; g < ng; ++g) {
        MangoPricingParams& p = gp[g];
        std::memset(&p, 0, sizeof(p));
        p.spot = 1.0;
        p.strike = 1.0;
        p.maturity = groups[g].T;
        p.volatility = groups[g].sigma;
        p.rate_const = groups[g].rep->rate_const;
        p.tenor_points = groups[g].rep->tenor_points;
        p.n_tenor_points = groups[g].rep->n_tenor_points;
        p.dividend_yield = groups[g].q;
        p.option_type = groups[g].type;
        Resolved& r = res[g];
        r.orig = static_cast<int32_t>(g);
        if (custom) {
          const std::string m = resolve_custom(p, &r);
          if (!m.empty()) throw std::invalid_argument(m);
        } else {
          std::vector<const MangoPricingParams*> one{&gp[g]};
          estimate_batch_grid(one, acc, &r.spec, &r.nt);
        }
        r.tv = time_varying(p);
      }
      b = create_batch_resolved(ctx, gp.data(), std::move(res),
                                std::vector<std::string>(static_cast<size_t>(ng)), trbdf2);
      run_batch(b);
      // Group results (statuses, grid sizes) and the context stats.
      std::vector<MangoGpuAmericanOut> gout(static_cast<size_t>(ng));
      std::string gmsg;
      fetch_batch(b, gout.data(), &gmsg);
      // sorted position of each group
      std::vector<int32_t> pos(static_cast<size_t>(ng), -1);
      for (size_t s = 0; s < b->order.size(); ++s) pos[b->order[s]] = static_cast<int32_t>(s);
      std::vector<int32_t> grp;
      std::vector<double> spot, strike;
      std::vector<int64_t> idx;
      for (int64_t i = 0; i < nn; ++i) {
        if (!valid[i]) continue;
        grp.push_back(pos[gof[i]]);
        spot.push_back(params[i].spot);
        strike.push_back(params[i].strike);
        idx.push_back(i);
      }
      const int64_t nout = static_cast<int64_t>(idx.size());
      if (nout > 0) {
        cudaStream_t st = ctx->stream;
        int nmax = 3;
        for (const Resolved& r : b->res) nmax = std::max(nmax, static_cast<int>(r.spec.n));
        int32_t* dg = static_cast<int32_t*>(d_grp.get(sizeof(int32_t) * nout));
        double* ds = static_cast<double*>(d_spot.get(sizeof(double) * nout));
        double* dk = static_cast<double*>(d_strike.get(sizeof(double) * nout));
        double* dscr = static_cast<double*>(d_scratch.get(sizeof(double) * 2 * nmax * nout));
        double* dout = static_cast<double*>(d_out.get(sizeof(double) * 4 * nout));
        check(cudaMemcpyAsync(dg, grp.data(), sizeof(int32_t) * nout, cudaMemcpyHostToDevice, st), "H2D");
        check(cudaMemcpyAsync(ds, spot.data(), sizeof(double) * nout, cudaMemcpyHostToDevice, st), "H2D");
        check(cudaMemcpyAsync(dk, strike.data(), sizeof(double) * nout, cudaMemcpyHostToDevice, st), "H2D");
        const int tb = 128;
        chain_outputs_kernel<<<static_cast<int>((nout + tb - 1) / tb), tb, 0, st>>>(
            static_cast<int>(nout), dg, ds, dk, b->d_tiles.as<TileDev>(), b->d_opts.as<OptDev>(),
            b->d_xs.as<double>(), b->d_pool.as<double>(), b->d_mode.as<int32_t>(),
            b->d_status.as<int32_t>(), b->mc, dscr, nmax, dout);
        check(cudaGetLastError(), "chain_outputs_kernel launch");
        std::vector<double> h(static_cast<size_t>(4 * nout));
        check(cudaMemcpyAsync(h.data(), dout, sizeof(double) * 4 * nout, cudaMemcpyDeviceToHost, st), "D2H");
        check(cudaStreamSynchronize(st), "stream synchronize");
        ctx->stats.kernel_launches += 1;
        for (int64_t j = 0; j < nout; ++j) {
          MangoGpuAmericanOut& o = out[idx[j]];
          const MangoGpuAmericanOut& go = gout[static_cast<size_t>(gof[idx[j]])];
          o.value = h[4 * j];
          o.delta = h[4 * j + 1];
          o.gamma = h[4 * j + 2];
          o.theta = h[4 * j + 3];
          o.status = go.status;
          o.n_space = go.n_space;
          o.n_time = go.n_time;
        }
      }
    } else {
      // Regular batch on one shared grid.
      GridSpec spec;
      int64_t nt = 0;
      if (custom) {
        // resolve_grid for the first option; the shared step count is that
        // time domain's (an explicit n_time, or the estimate's own steps).
        Resolved r;
        const std::string m = resolve_custom(params[0], &r);
        if (!m.empty()) throw std::invalid_argument(m);
        spec = r.spec;
        const int32_t k = custom_grid->kind;
        const bool explicit_nt = k == MANGO_GPU_GRID_SINH || k == MANGO_GPU_GRID_UNIFORM ||
                                 ((k == MANGO_GPU_GRID_FIXED_N || k == MANGO_GPU_GRID_FIXED_N_AT_VOL) &&
                                  custom_grid->n_time > 0);
        nt = explicit_nt ? custom_grid->n_time : r.nt;
      } else {
        std::vector<const MangoPricingParams*> ps;
        for (int64_t i = 0; i < nn; ++i)
          if (valid[i]) ps.push_back(&params[i]);
        if (!ps.empty()) estimate_batch_grid(ps, acc, &spec, &nt);
      }
      std::vector<Resolved> res(static_cast<size_t>(nn));
      std::vector<double> taus;
      for (int64_t i = 0; i < nn; ++i) {
        res[i].orig = static_cast<int32_t>(i);
        res[i].spec = spec;
        res[i].nt = nt;
        if (!valid[i]) {
          res[i].status = MANGO_ERR_VALIDATION;
          continue;
        }
        // PDEGridConfig{shared spec, shared n_steps, this option's dividend
        // times} (american_option_batch.cpp:447-470).
        const MangoPricingParams& p = params[i];
        res[i].tv = time_varying(p);
        taus.clear();
        for (uint64_t j = 0; j < p.n_dividends; ++j) {
          const double tau = p.maturity - p.dividends[j].calendar_time;
          if (tau > 0.0 && tau < p.maturity) taus.push_back(tau);
        }
        explicit_time_domain(p.maturity, nt, taus, &res[i]);
      }
      b = create_batch_resolved(ctx, params, std::move(res), vmsg, trbdf2);
      run_batch(b);
      std::string fm;
      fetch_batch(b, out, &fm);
    }
    uint64_t failed = 0;
    for (int64_t i = 0; i < nn; ++i) {
      failed += out[i].status != MANGO_OK;
      if (out[i].status != MANGO_OK && first_err.empty())
        first_err = vmsg[i].empty() ? "solver failure" : vmsg[i];
    }
    if (out_failed) *out_failed = failed;
    if (failed && err) set_err(err, MANGO_OK, first_err);
    release();
    return MANGO_OK;
  } catch (const std::invalid_argument& e) {
    release();
    set_err(err, MANGO_ERR_VALIDATION, e.what());
    return MANGO_ERR_VALIDATION;
  } catch (const std::exception& e) {
    release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}
