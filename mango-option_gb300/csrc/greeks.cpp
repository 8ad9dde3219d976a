// greeks.cpp -- batched bump-and-reprice sensitivities on a frozen grid.
//
// The reference's FDM result exposes value, delta, gamma and theta only
// (src/option/american_option_result.cpp:25-121); sensitivities to
// volatility, rate, dividend yield and strike are obtained by central
// differences of the solver on a fixed grid.  Each option's grid is resolved
// once (resolve_grid, src/option/american_option.cpp:54-73) and the eight
// bumped copies are priced on exactly that grid (the log-moneyness grid is
// independent of the strike, so a strike bump only moves x = ln(S/K)), all in
// one device batch.  Options with a yield curve or discrete dividends take
// the time-varying march like their unbumped price; for a yield curve the
// rate bump is a parallel shift of the continuously compounded zero rates
// (every log discount ln D(t) moves by -h t).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"

using namespace mgpu;

extern "C" MangoStatus mango_gpu_price_american_greeks_batch(
    MangoGpuContext* ctx, const MangoPricingParams* params, uint64_t n, const MangoGpuGrid* grids,
    uint64_t grid_stride, double h_rel, MangoGpuGreeksOut* out, uint64_t* out_failed,
    MangoError* err) {
  if (!ctx || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, params or out");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 26)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^26 options");
    return MANGO_ERR_VALIDATION;
  }
  const double h = h_rel > 0.0 ? h_rel : 1e-5;
  MangoGpuBatch* b = nullptr;
  try {
    const int64_t nn = static_cast<int64_t>(n);
    std::vector<Resolved> base(static_cast<size_t>(nn));
    std::vector<std::string> msg(static_cast<size_t>(nn));
    parallel_for(nn, [&](int64_t i) {
      thread_local std::vector<double> scratch;
      base[i].orig = static_cast<int32_t>(i);
      std::string m = validate(params[i], true);
      if (m.empty()) {
        MangoGpuGrid g{};
        g.kind = MANGO_GPU_GRID_AUTO;
        if (grids) g = grids[grid_stride ? i : 0];
        m = resolve(params[i], g, &base[i], &scratch);
      }
      if (!m.empty()) {
        base[i].status = MANGO_ERR_VALIDATION;
        msg[i] = m;
      }
    });
    // Copies: 0 base, then (+,-) for volatility, rate, dividend yield, strike.
    constexpr int kCopies = 9;
    std::vector<MangoPricingParams> pp(static_cast<size_t>(kCopies * nn));
    std::vector<Resolved> res(static_cast<size_t>(kCopies * nn));
    std::vector<double> step(static_cast<size_t>(4 * nn), 0.0);
    // Shifted curves of the rate bumps, alive until the batch is packed.
    std::vector<std::vector<MangoTenorPoint>> shifted(static_cast<size_t>(2 * nn));
    for (int64_t i = 0; i < nn; ++i) {
      const MangoPricingParams& p = params[i];
      const double hv = h * p.volatility;
      const double hr = h * std::max(std::fabs(p.rate_const), 1e-2);
      const double hq = h * std::max(p.dividend_yield, 1e-2);
      const double hk = h * p.strike;
      step[4 * i + 0] = hv;
      step[4 * i + 1] = hr;
      step[4 * i + 2] = hq;
      step[4 * i + 3] = hk;
      for (int c = 0; c < kCopies; ++c) {
        MangoPricingParams q = p;
        const double sgn = (c % 2 == 1) ? 1.0 : -1.0;
        switch ((c + 1) / 2) {
          case 1: q.volatility += sgn * hv; break;
          case 2:
            if (q.n_tenor_points != 0 && base[i].status == 0) {
              std::vector<MangoTenorPoint>& v = shifted[static_cast<size_t>((c - 3) * nn + i)];
              v.assign(q.tenor_points, q.tenor_points + q.n_tenor_points);
              for (auto& t : v) t.log_discount -= sgn * hr * t.tenor;
              q.tenor_points = v.data();
            } else {
              q.rate_const += sgn * hr;
            }
            break;
          case 3: q.dividend_yield = std::max(0.0, q.dividend_yield + sgn * hq); break;
          case 4: q.strike += sgn * hk; break;
          default: break;
        }
        const size_t j = static_cast<size_t>(c * nn + i);
        pp[j] = q;
        res[j] = base[i];
        res[j].orig = static_cast<int32_t>(j);
      }
      // A dividend-yield bump clipped at zero is one-sided: record the actual
      // step so the difference quotient stays correct.
      step[4 * i + 2] = pp[static_cast<size_t>(5 * nn + i)].dividend_yield -
                        pp[static_cast<size_t>(6 * nn + i)].dividend_yield;
    }
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    b = create_batch_resolved(ctx, pp.data(), std::move(res),
                              std::vector<std::string>(static_cast<size_t>(kCopies * nn)), nullptr);
    run_batch(b);
    std::vector<MangoGpuAmericanOut> o(static_cast<size_t>(kCopies * nn));
    std::string first;
    fetch_batch(b, o.data(), &first);
    destroy_batch(b);
    b = nullptr;
    uint64_t failed = 0;
    for (int64_t i = 0; i < nn; ++i) {
      MangoGpuGreeksOut& g = out[i];
      std::memset(&g, 0, sizeof(g));
      g.base = o[static_cast<size_t>(i)];
      g.base.status = base[i].status != 0 ? base[i].status : g.base.status;
      bool ok = g.base.status == MANGO_OK;
      for (int c = 1; c < kCopies && ok; ++c) ok = o[static_cast<size_t>(c * nn + i)].status == MANGO_OK;
      if (!ok && g.base.status == MANGO_OK) g.base.status = MANGO_ERR_SOLVER;
      auto cd = [&](int k) {
        const double up = o[static_cast<size_t>((2 * k + 1) * nn + i)].value;
        const double dn = o[static_cast<size_t>((2 * k + 2) * nn + i)].value;
        return (up - dn) / (2.0 * step[4 * i + k]);
      };
      if (ok) {
        g.vega = cd(0);
        g.rho = cd(1);
        g.dividend_rho = (o[static_cast<size_t>(5 * nn + i)].value - o[static_cast<size_t>(6 * nn + i)].value) /
                         step[4 * i + 2];
        g.dstrike = cd(3);
      } else {
        g.vega = g.rho = g.dividend_rho = g.dstrike = NAN;
        if (first.empty()) first = msg[i];
      }
      failed += g.base.status != MANGO_OK;
    }
    if (out_failed) *out_failed = failed;
    if (failed && err) set_err(err, MANGO_OK, first.empty() ? "solver failure" : first);
    return MANGO_OK;
  } catch (const std::exception& e) {
    if (b) destroy_batch(b);
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}
