// iv.cu -- batched FDM implied volatility on the GPU.
//
// Restates IVSolver::solve / solve_brent (src/option/iv_solver.cpp:133-242)
// with brent_find_root (src/math/root_finding.hpp:145-302) as a per-quote
// state machine on the device.  Every quote keeps its own fixed grid; each
// Brent evaluation re-prices all still-active quotes at their current trial
// volatility with the same setup / march / value kernels as batched pricing,
// then one thread per quote advances Brent by exactly one function value.
// The per-iteration launch sequence is captured once as a CUDA graph and
// replayed until every quote has converged or failed.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"

namespace mgpu {

// Brent state of one quote (root_finding.hpp:145-302 variables).
struct BrentDev {
  double a, b, c, d, fa, fb, fc, s;
  double root, ferr;
  int32_t iter, mflag, phase, code;  // phase: 0 eval a, 1 eval b, 2 eval s, 3 done
};

// Result codes of the state machine.
constexpr int32_t kIvOk = 0, kIvBracket = 1, kIvMaxIter = 2, kIvNumerical = 3;

__global__ void brent_init_kernel(int m, const double* __restrict__ upper, BrentDev* __restrict__ S,
                                  double* __restrict__ sigma, int32_t* __restrict__ active) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  BrentDev s{};
  s.a = 0.01;  // IVSolver::solve_brent vol_lower (iv_solver.cpp:150)
  s.b = upper[k];
  s.phase = 0;
  S[k] = s;
  sigma[k] = s.a;
  active[k] = 1;
}

namespace {

__device__ __forceinline__ void swap_d(double& x, double& y) {
  const double t = x;
  x = y;
  y = t;
}

// Convergence test and next trial point at the top of a Brent iteration;
// returns false when the quote is finished.
__device__ bool brent_propose(BrentDev& s, double tol, int max_iter) {
  if (s.iter >= max_iter) {
    s.code = kIvMaxIter;
    s.root = s.b;
    s.ferr = fabs(s.fb);
    return false;
  }
  if (fabs(s.fb) < tol || fabs(s.b - s.a) < tol) {
    s.code = kIvOk;
    s.root = s.b;
    s.ferr = fabs(s.fb);
    s.iter += 1;  // the reference reports iter + 1 here
    return false;
  }
  const double a = s.a, b = s.b, c = s.c, fa = s.fa, fb = s.fb, fc = s.fc;
  double x;
  if (fa != fc && fb != fc) {  // inverse quadratic interpolation
    x = a * fb * fc / ((fa - fb) * (fa - fc)) + b * fa * fc / ((fb - fa) * (fb - fc)) +
        c * fa * fb / ((fc - fa) * (fc - fb));
  } else {  // secant
    x = b - fb * (b - a) / (fb - fa);
  }
  const double bis = (3.0 * a + b) / 4.0;
  const bool c1 = !((x > bis && x < b) || (x < bis && x > b));
  const bool c2 = s.mflag && fabs(x - b) >= fabs(b - c) / 2.0;
  const bool c3 = !s.mflag && fabs(x - b) >= fabs(c - s.d) / 2.0;
  const bool c4 = s.mflag && fabs(b - c) < tol;
  const bool c5 = !s.mflag && fabs(c - s.d) < tol;
  if (c1 || c2 || c3 || c4 || c5) {
    x = (a + b) / 2.0;
    s.mflag = 1;
  } else {
    s.mflag = 0;
  }
  s.s = x;
  return true;
}

}  // namespace

// Consume the objective value at the last trial point and advance Brent.
// f = value_at(spot) - market price (iv_solver.cpp:48-119); a failed march
// gives NaN, as the reference's objective does.
__global__ void brent_step_kernel(int m, BrentDev* __restrict__ S, const double* __restrict__ out4,
                                  const int32_t* __restrict__ mstatus,
                                  const double* __restrict__ price, double* __restrict__ sigma,
                                  int32_t* __restrict__ active, double tol, int max_iter,
                                  int* __restrict__ n_active) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= m) return;
  BrentDev s = S[k];
  if (s.phase == 3) {
    active[k] = 0;
    return;
  }
  const double f = mstatus[k] == kStatusOk ? out4[4 * static_cast<size_t>(k)] - price[k]
                                           : __longlong_as_double(0x7ff8000000000000ll);
  bool go = true;
  double next = 0.0;
  if (s.phase == 0) {
    s.fa = f;
    s.phase = 1;
    next = s.b;
  } else if (s.phase == 1) {
    s.fb = f;
    if (!isfinite(s.fa) || !isfinite(s.fb)) {
      s.code = kIvNumerical;
      s.ferr = __longlong_as_double(0x7ff8000000000000ll);
      s.iter = 0;
      go = false;
    } else if (s.fa * s.fb > 0.0) {
      s.code = kIvBracket;
      s.ferr = fmin(fabs(s.fa), fabs(s.fb));
      s.iter = 0;
      go = false;
    } else if (fabs(s.fa) < tol) {
      s.code = kIvOk;
      s.root = s.a;
      s.ferr = fabs(s.fa);
      s.iter = 0;
      go = false;
    } else if (fabs(s.fb) < tol) {
      s.code = kIvOk;
      s.root = s.b;
      s.ferr = fabs(s.fb);
      s.iter = 0;
      go = false;
    } else {
      if (fabs(s.fa) < fabs(s.fb)) {
        swap_d(s.a, s.b);
        swap_d(s.fa, s.fb);
      }
      s.c = s.a;
      s.fc = s.fa;
      s.mflag = 1;
      s.d = 0.0;
      s.iter = 0;
      go = brent_propose(s, tol, max_iter);
      next = s.s;
      s.phase = 2;
    }
  } else {
    const double fs = f;
    if (!isfinite(fs)) {
      s.code = kIvNumerical;
      s.root = s.s;
      s.ferr = __longlong_as_double(0x7ff8000000000000ll);
      s.iter += 1;
      go = false;
    } else {
      s.d = s.c;
      s.c = s.b;
      s.fc = s.fb;
      if (s.fa * fs < 0.0) {
        s.b = s.s;
        s.fb = fs;
      } else {
        s.a = s.s;
        s.fa = fs;
      }
      if (fabs(s.fa) < fabs(s.fb)) {
        swap_d(s.a, s.b);
        swap_d(s.fa, s.fb);
      }
      s.iter += 1;
      go = brent_propose(s, tol, max_iter);
      next = s.s;
    }
  }
  if (!go) {
    s.phase = 3;
    active[k] = 0;
  } else {
    sigma[k] = next;
    atomicAdd(n_active, 1);
  }
  S[k] = s;
}

namespace {

// validate_iv_query (src/option/option_spec.cpp:52-112) plus the engine's
// scope; returns the MangoStatus and a message.
int32_t validate_query(const MangoIvQuery& q, std::string* msg) {
  auto bad = [&](int32_t code, const char* m) {
    *msg = m;
    return code;
  };
  if (!(q.spot > 0.0) || !std::isfinite(q.spot)) return bad(MANGO_ERR_VALIDATION, "invalid spot");
  if (!(q.strike > 0.0) || !std::isfinite(q.strike)) return bad(MANGO_ERR_VALIDATION, "invalid strike");
  if (!(q.maturity > 0.0) || !std::isfinite(q.maturity))
    return bad(MANGO_ERR_VALIDATION, "invalid maturity");
  if (!std::isfinite(q.rate_const)) return bad(MANGO_ERR_VALIDATION, "invalid rate");
  if (q.dividend_yield < 0.0 || !std::isfinite(q.dividend_yield))
    return bad(MANGO_ERR_VALIDATION, "invalid dividend yield");
  if (q.option_type != MANGO_PUT && q.option_type != MANGO_CALL)
    return bad(MANGO_ERR_VALIDATION, "invalid option type");
  if (q.n_tenor_points != 0) return bad(MANGO_ERR_VALIDATION, "yield curves are not supported by the GPU engine");
  if (q.n_dividends != 0) return bad(MANGO_ERR_VALIDATION, "discrete dividends are not supported by the GPU engine");
  if (!std::isfinite(q.market_price) || q.market_price <= 0.0)
    return bad(MANGO_ERR_VALIDATION, "invalid market price");
  const bool put = q.option_type == MANGO_PUT;
  const double intrinsic = put ? std::max(q.strike - q.spot, 0.0) : std::max(q.spot - q.strike, 0.0);
  const double upper = put ? q.strike : q.spot;
  if (q.market_price < intrinsic) return bad(MANGO_ERR_ARBITRAGE, "market price below intrinsic value");
  if (q.market_price > upper) return bad(MANGO_ERR_ARBITRAGE, "market price above the upper bound");
  return MANGO_OK;
}

}  // namespace
}  // namespace mgpu

using namespace mgpu;

extern "C" MangoStatus mango_gpu_solve_iv_batch(MangoGpuContext* ctx, const MangoIvQuery* queries,
                                                uint64_t n, const MangoGpuGrid* grids,
                                                uint64_t grid_stride, const MangoIvConfig* config,
                                                MangoIvBatchSlot* out, uint64_t* out_failed,
                                                MangoError* err) {
  if (!ctx || (n > 0 && (!queries || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, queries or out");
    return MANGO_ERR_VALIDATION;
  }
  if (!grids) {
    set_err(err, MANGO_ERR_VALIDATION,
            "IV needs a fixed grid per quote (MANGO_GPU_GRID_FIXED_N_AT_VOL, _SINH or _UNIFORM)");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 30)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^30 quotes");
    return MANGO_ERR_VALIDATION;
  }
  const double tol = (config && config->brent_tol_abs > 0.0) ? config->brent_tol_abs : 1e-6;
  const int max_iter = (config && config->max_iter > 0) ? config->max_iter : 100;
  MangoGpuBatch* b = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
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
      p.option_type = q.option_type;
      p.volatility = 0.2;  // placeholder; every evaluation overrides it
      vstatus[i] = validate_query(q, &vmsg[i]);
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
    b = create_batch(ctx, pp.data(), nn, grids, grid_stride, nullptr);
    const int64_t m = static_cast<int64_t>(b->order.size());
    std::vector<int32_t> code(static_cast<size_t>(m), kIvNumerical);
    std::vector<BrentDev> hs(static_cast<size_t>(m));
    if (m > 0) {
      cudaStream_t st = ctx->stream;
      std::vector<double> hi_sorted(static_cast<size_t>(m)), px(static_cast<size_t>(m));
      for (int64_t s = 0; s < m; ++s) {
        hi_sorted[s] = upper[b->order[s]];
        px[s] = queries[b->order[s]].market_price;
      }
      DevBuf d_state, d_sigma, d_active, d_hi, d_px, d_count;
      HostBuf h_count;
      BrentDev* S = static_cast<BrentDev*>(d_state.get(sizeof(BrentDev) * m));
      double* sigma = static_cast<double*>(d_sigma.get(sizeof(double) * m));
      int32_t* active = static_cast<int32_t*>(d_active.get(sizeof(int32_t) * m));
      double* dhi = static_cast<double*>(d_hi.get(sizeof(double) * m));
      double* dpx = static_cast<double*>(d_px.get(sizeof(double) * m));
      int* count = static_cast<int*>(d_count.get(sizeof(int) * 4));
      int* hcount = static_cast<int*>(h_count.get(sizeof(int) * 4));
      check(cudaMemcpyAsync(dhi, hi_sorted.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dpx, px.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
      const int tb = 256, gb = static_cast<int>((m + tb - 1) / tb);
      brent_init_kernel<<<gb, tb, 0, st>>>(static_cast<int>(m), dhi, S, sigma, active);
      check(cudaGetLastError(), "brent_init launch");

      MarchConst mc = b->mc;
      mc.value_only = 1;
      mc.sigma = sigma;
      mc.active = active;
      const int ntiles = b->ntiles;
      const int threads = ntiles * kTile;
      const int blocks = std::max(1, std::min<int>(ctx->num_sms * ctx->march_blocks_per_sm, (ntiles + 3) / 4));
      // One Brent evaluation as a graph: reset counters, setup, march,
      // value, Brent update.
      check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "begin capture");
      cudaMemsetAsync(b->d_queue.p, 0, sizeof(int) * 4, st);
      cudaMemsetAsync(count, 0, sizeof(int) * 4, st);
      prep_kernel<<<(threads + 127) / 128, 128, 0, st>>>(b->d_tiles.as<TileDev>(), ntiles,
                                                         b->d_opts.as<OptDev>(), b->d_xs.as<double>(),
                                                         b->d_pool.as<double>(), b->d_flags.as<uint8_t>(),
                                                         b->d_mode.as<int32_t>(), mc);
      march_kernel<<<blocks, 128, 0, st>>>(b->d_tiles.as<TileDev>(), ntiles, b->d_opts.as<OptDev>(),
                                           b->d_pool.as<double>(), b->d_flags.as<uint8_t>(),
                                           b->d_mode.as<int32_t>(), b->d_status.as<int32_t>(),
                                           b->d_queue.as<int>(), mc);
      outputs_kernel<<<(threads + 127) / 128, 128, 0, st>>>(
          b->d_tiles.as<TileDev>(), ntiles, b->d_opts.as<OptDev>(), b->d_xs.as<double>(),
          b->d_pool.as<double>(), b->d_mode.as<int32_t>(), b->d_status.as<int32_t>(), mc,
          b->d_out4.as<double>());
      brent_step_kernel<<<gb, tb, 0, st>>>(static_cast<int>(m), S, b->d_out4.as<double>(),
                                           b->d_status.as<int32_t>(), dpx, sigma, active, tol,
                                           max_iter, count);
      cudaMemcpyAsync(hcount, count, sizeof(int), cudaMemcpyDeviceToHost, st);
      check(cudaStreamEndCapture(st, &graph), "end capture");
      check(cudaGraphInstantiate(&exec, graph, 0), "graph instantiate");
      // Two endpoint evaluations plus at most max_iter Brent steps.
      int launches = 0;
      for (int it = 0; it < max_iter + 3; ++it) {
        check(cudaGraphLaunch(exec, st), "graph launch");
        check(cudaStreamSynchronize(st), "stream synchronize");
        ++launches;
        if (hcount[0] == 0) break;
      }
      ctx->stats.kernel_launches = 4LL * launches + 1;
      check(cudaMemcpyAsync(hs.data(), S, sizeof(BrentDev) * m, cudaMemcpyDeviceToHost, st), "D2H state");
      check(cudaStreamSynchronize(st), "stream synchronize");
      cudaGraphExecDestroy(exec);
      exec = nullptr;
      cudaGraphDestroy(graph);
      graph = nullptr;
      for (DevBuf* d : {&d_state, &d_sigma, &d_active, &d_hi, &d_px, &d_count}) d->release();
      h_count.release();
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
      const BrentDev& r = hs[s];
      MangoIvBatchSlot& o = out[b->order[s]];
      switch (r.code) {
        case kIvOk: o.status = MANGO_OK; break;
        case kIvBracket: o.status = MANGO_ERR_BRACKETING; break;
        case kIvMaxIter: o.status = MANGO_ERR_NO_CONVERGENCE; break;
        default: o.status = MANGO_ERR_SOLVER; break;
      }
      o.success.implied_vol = r.code == kIvOk ? r.root : NAN;
      o.success.iterations = static_cast<uint64_t>(r.iter);
      o.success.final_error = r.ferr;
      o.success.vega = 0.0;
      o.success.has_vega = 0;
      o.success.used_rate_approximation = 0;
    }
    for (int64_t i = 0; i < nn; ++i) failed += out[i].status != MANGO_OK;
    if (out_failed) *out_failed = failed;
    if (failed && err) set_err(err, MANGO_OK, first.empty() ? "root finding failed" : first);
    destroy_batch(b);
    return MANGO_OK;
  } catch (const std::exception& e) {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (b) destroy_batch(b);
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}
