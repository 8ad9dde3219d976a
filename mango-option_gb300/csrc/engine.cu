// engine.cu -- C ABI implementation (include/mango_gpu.h) and the batched
// pricing pipeline.  Mirrors the reference's ABI conventions: status codes
// and 256-byte messages (src/ffi/mango_c_api.cpp:23-31), every exception
// caught at the boundary (mango_c_api.cpp:354-360), per-slot status for batch
// calls (mango_c_api.cpp:523-576).
#include "engine.hpp"
#include "wmarch.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <queue>
#include <thread>
#include <utility>

namespace mgpu {

__global__ void fp64_probe_kernel(double* out, int iters);

void check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    throw CudaError(std::string(what) + ": " + cudaGetErrorName(e) + " (" +
                    cudaGetErrorString(e) + ")");
  }
}

void* DevBuf::get(size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes > cap) {
    if (p) check(cudaFree(p), "cudaFree");
    p = nullptr;
    cap = 0;
    check(cudaMalloc(&p, bytes), "cudaMalloc");
    cap = bytes;
  }
  return p;
}
void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}
void* HostBuf::get(size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes > cap) {
    if (p) check(cudaFreeHost(p), "cudaFreeHost");
    p = nullptr;
    cap = 0;
    check(cudaMallocHost(&p, bytes), "cudaMallocHost");
    cap = bytes;
  }
  return p;
}
void HostBuf::release() {
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
}

void parallel_for(int64_t n, const std::function<void(int64_t)>& f, int64_t grain) {
  const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  const int64_t per = std::max<int64_t>(1, grain);
  const int64_t nth = std::min<int64_t>(hw, (n + per - 1) / per);
  if (nth <= 1) {
    for (int64_t i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(static_cast<size_t>(nth));
  for (int64_t t = 0; t < nth; ++t) {
    th.emplace_back([&, t] {
      const int64_t a = n * t / nth, b = n * (t + 1) / nth;
      for (int64_t i = a; i < b; ++i) f(i);
    });
  }
  for (auto& x : th) x.join();
}

std::string schedule_error(const MangoTenorPoint* tenor_points, uint64_t n_tenor_points,
                           const MangoDividend* dividends, uint64_t n_dividends, double maturity) {
  if (n_tenor_points != 0) {
    // build_rate + YieldCurve::from_points (src/ffi/mango_c_api.cpp:44-64,
    // src/option/yield_curve.hpp): sorted by tenor, the first at t = 0 with
    // log discount 0, tenors strictly increasing.  Non-finite entries are
    // rejected too.
    if (!tenor_points) return "tenor_points is null but n_tenor_points > 0";
    std::vector<MangoTenorPoint> pts(tenor_points, tenor_points + n_tenor_points);
    for (const auto& t : pts)
      if (!std::isfinite(t.tenor) || !std::isfinite(t.log_discount))
        return "invalid yield curve: non-finite tenor point";
    std::sort(pts.begin(), pts.end(),
              [](const MangoTenorPoint& a, const MangoTenorPoint& b) { return a.tenor < b.tenor; });
    if (pts[0].tenor != 0.0) return "invalid yield curve: First point must have t=0";
    if (std::abs(pts[0].log_discount) > 1e-10)
      return "invalid yield curve: log_discount at t=0 must be 0";
    for (size_t i = 1; i < pts.size(); ++i)
      if (pts[i].tenor <= pts[i - 1].tenor + 1e-10)
        return "invalid yield curve: Tenors must be strictly increasing";
  }
  if (n_dividends != 0) {
    // build_dividends + validate_pricing_params / validate_iv_query
    // (src/option/option_spec.cpp:89-110, 131-153)
    if (!dividends) return "dividends is null but n_dividends > 0";
    for (uint64_t i = 0; i < n_dividends; ++i) {
      const MangoDividend& d = dividends[i];
      if (d.calendar_time < 0.0 || d.calendar_time > maturity) return "invalid dividend time";
      if (d.amount < 0.0) return "invalid dividend amount";
      if (!std::isfinite(d.calendar_time) || !std::isfinite(d.amount)) return "invalid dividend";
    }
  }
  return {};
}

std::string validate(const MangoPricingParams& p, bool allow_tv) {
  // validate_pricing_params (src/option/option_spec.cpp:8-40, 117-157)
  if (!(p.spot > 0.0) || !std::isfinite(p.spot)) return "invalid spot";
  if (!(p.strike > 0.0) || !std::isfinite(p.strike)) return "invalid strike";
  if (!(p.maturity > 0.0) || !std::isfinite(p.maturity)) return "invalid maturity";
  if (p.n_tenor_points == 0 && !std::isfinite(p.rate_const)) return "invalid rate";
  if (p.dividend_yield < 0.0 || !std::isfinite(p.dividend_yield)) return "invalid dividend yield";
  if (!(p.volatility > 0.0) || !std::isfinite(p.volatility)) return "invalid volatility";
  if (p.option_type != MANGO_PUT && p.option_type != MANGO_CALL) return "invalid option type";
  if (!allow_tv) {
    if (p.n_tenor_points != 0) return "yield curves are not supported by this entry point";
    if (p.n_dividends != 0) return "discrete dividends are not supported by this entry point";
    return {};
  }
  return schedule_error(p.tenor_points, p.n_tenor_points, p.dividends, p.n_dividends, p.maturity);
}

bool time_varying(const MangoPricingParams& p) {
  if (p.n_tenor_points != 0) return true;
  for (uint64_t i = 0; i < p.n_dividends; ++i) {
    const double tau = p.maturity - p.dividends[i].calendar_time;
    if (tau > 0.0 && tau < p.maturity) return true;
  }
  return false;
}

namespace {
// Times to expiry of the dividends inside (0, T) and their largest
// amount / strike (estimate_pde_grid, grid_spec_types.cpp:59-67, 96-103).
void dividend_taus(const MangoPricingParams& p, std::vector<double>* taus, double* max_dk) {
  taus->clear();
  *max_dk = 0.0;
  for (uint64_t i = 0; i < p.n_dividends; ++i) {
    const double tau = p.maturity - p.dividends[i].calendar_time;
    if (tau > 0.0 && tau < p.maturity) {
      taus->push_back(tau);
      *max_dk = std::max(*max_dk, p.dividends[i].amount / p.strike);
    }
  }
}
}  // namespace

void explicit_time_domain(double maturity, int64_t n_time, const std::vector<double>& taus,
                          Resolved* r) {
  // resolve_grid for a PDEGridConfig (american_option.cpp:64-72)
  if (taus.empty()) {
    r->tp.clear();
    r->nt = n_time;
    return;
  }
  time_points(0.0, maturity, maturity / static_cast<double>(n_time), taus, &r->tp, &r->nt);
}

std::string resolve(const MangoPricingParams& p, const MangoGpuGrid& g, Resolved* r,
                    std::vector<double>* scratch) {
  // resolve_grid (src/option/american_option.cpp:54-73)
  const Accuracy def = default_accuracy();
  r->tv = time_varying(p);
  r->tp.clear();
  if (r->tv) {
    // Dividends widen the estimated grid and add mandatory time points; an
    // explicit grid takes them as the PDEGridConfig's mandatory times, as
    // BatchAmericanOptionSolver attaches them (american_option_batch.cpp:
    // 447-470).
    std::vector<double> taus;
    double max_dk = 0.0;
    dividend_taus(p, &taus, &max_dk);
    switch (g.kind) {
      case MANGO_GPU_GRID_AUTO:
        estimate_grid_div(p.spot, p.strike, p.maturity, p.volatility, def, taus, max_dk, &r->spec,
                          &r->nt, &r->tp, scratch);
        break;
      case MANGO_GPU_GRID_FIXED_N:
      case MANGO_GPU_GRID_FIXED_N_AT_VOL: {
        if (g.n_space < 3 || g.n_time < 0) return "grid: n_space >= 3 and n_time >= 0 required";
        const double vol = g.kind == MANGO_GPU_GRID_FIXED_N ? p.volatility : g.alpha;
        if (!(vol > 0.0) || !std::isfinite(vol)) return "grid: sizing volatility must be > 0";
        Accuracy a = def;
        a.min_points = a.max_points = g.n_space;
        estimate_grid_div(p.spot, p.strike, p.maturity, vol, a, taus, max_dk, &r->spec, &r->nt,
                          &r->tp, scratch);
        if (g.n_time > 0) explicit_time_domain(p.maturity, g.n_time, taus, r);
        break;
      }
      case MANGO_GPU_GRID_SINH:
      case MANGO_GPU_GRID_UNIFORM:
        if (g.n_space < 3 || g.n_time < 1) return "grid: n_space >= 3 and n_time >= 1 required";
        if (!(g.x_min < g.x_max)) return "grid: x_min < x_max required";
        if (g.kind == MANGO_GPU_GRID_SINH && !(g.alpha > 0.0)) return "grid: alpha > 0 required";
        r->spec = g.kind == MANGO_GPU_GRID_SINH ? sinh_spec(g.x_min, g.x_max, g.n_space, g.alpha)
                                                : uniform_spec(g.x_min, g.x_max, g.n_space);
        explicit_time_domain(p.maturity, g.n_time, taus, r);
        break;
      default:
        return "grid: unknown kind";
    }
    if (r->spec.n > 100000) return "grid: n_space above 100000";
    if (r->nt > 100000000 || r->nt < 1) return "grid: n_time outside [1, 1e8]";
    return {};
  }
  switch (g.kind) {
    case MANGO_GPU_GRID_AUTO:
      estimate_grid(p.spot, p.strike, p.maturity, p.volatility, def, &r->spec, &r->nt, scratch);
      break;
    case MANGO_GPU_GRID_FIXED_N:
    case MANGO_GPU_GRID_FIXED_N_AT_VOL: {
      if (g.n_space < 3 || g.n_time < 0) return "grid: n_space >= 3 and n_time >= 0 required";
      const double vol = g.kind == MANGO_GPU_GRID_FIXED_N ? p.volatility : g.alpha;
      if (!(vol > 0.0) || !std::isfinite(vol)) return "grid: sizing volatility must be > 0";
      Accuracy a = def;
      a.min_points = a.max_points = g.n_space;
      if (g.n_time > 0) {
        estimate_spec(p.spot, p.strike, p.maturity, vol, a, &r->spec);
        r->nt = g.n_time;
      } else {
        // n_time 0: the estimate's own step count (GridAccuracyParams alone)
        estimate_grid(p.spot, p.strike, p.maturity, vol, a, &r->spec, &r->nt, scratch);
      }
      break;
    }
    case MANGO_GPU_GRID_SINH:
      if (g.n_space < 3 || g.n_time < 1) return "grid: n_space >= 3 and n_time >= 1 required";
      if (!(g.x_min < g.x_max)) return "grid: x_min < x_max required";
      if (!(g.alpha > 0.0)) return "grid: alpha > 0 required";
      r->spec = sinh_spec(g.x_min, g.x_max, g.n_space, g.alpha);
      r->nt = g.n_time;
      break;
    case MANGO_GPU_GRID_UNIFORM:
      if (g.n_space < 3 || g.n_time < 1) return "grid: n_space >= 3 and n_time >= 1 required";
      if (!(g.x_min < g.x_max)) return "grid: x_min < x_max required";
      r->spec = uniform_spec(g.x_min, g.x_max, g.n_space);
      r->nt = g.n_time;
      break;
    default:
      return "grid: unknown kind";
  }
  if (r->spec.n > 100000) return "grid: n_space above 100000";
  if (r->nt > 100000000) return "grid: n_time above 1e8";
  return {};
}

void set_err(MangoError* err, int32_t code, const std::string& msg) {
  if (!err) return;
  err->code = code;
  std::snprintf(err->message, sizeof(err->message), "%s", msg.c_str());
}

namespace {
using Clock = std::chrono::steady_clock;
double ms_since(Clock::time_point t0) {
  return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}
}  // namespace

MarchConst make_const(const MangoGpuTrbdf2* trbdf2) {
  MarchConst mc{};
  mc.gamma = (trbdf2 && trbdf2->gamma > 0.0) ? trbdf2->gamma : 2.0 - std::sqrt(2.0);
  mc.rannacher = trbdf2 ? (trbdf2->rannacher_startup != 0) : 1;
  // solve_stage2 coefficients (pde_solver.hpp:372-380)
  const double omg = 1.0 - mc.gamma, tmg = 2.0 - mc.gamma, den = mc.gamma * tmg;
  mc.alpha = 1.0 / den;
  mc.beta = -(omg * omg) / den;
  return mc;
}

void destroy_batch(MangoGpuBatch* b) {
  if (!b) return;
  for (mgpu::DevBuf* d : {&b->d_handoff, &b->d_pool, &b->d_xs, &b->d_grids, &b->d_flags, &b->d_opts, &b->d_tiles, &b->d_mode,
                          &b->d_status, &b->d_out4, &b->d_queue, &b->d_tv, &b->d_tv_tp,
                          &b->d_tv_curve, &b->d_tv_ev, &b->d_wt, &b->d_tile_warp, &b->d_bins,
                          &b->d_bin_cnt, &b->d_tile_done})
    d->release();
  for (mgpu::HostBuf* h : {&b->h_xs, &b->h_grids, &b->h_opts, &b->h_tiles, &b->h_out4, &b->h_status})
    h->release();
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : b->run_ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : b->wev)
    if (e) cudaEventDestroy(e);
  if (b->wstream) {
    cudaStreamSynchronize(b->wstream);
    cudaStreamDestroy(b->wstream);
  }
  delete b;
}

// Validate, resolve grids, sort/tile, pack and upload.
MangoGpuBatch* create_batch(MangoGpuContext* ctx, const MangoPricingParams* params, int64_t n,
                            const MangoGpuGrid* grids, uint64_t grid_stride,
                            const MangoGpuTrbdf2* trbdf2, MangoGpuBatch* reuse,
                            cudaStream_t stream) {
  auto t0 = Clock::now();
  std::vector<Resolved> res(static_cast<size_t>(n));
  std::vector<std::string> msgs(static_cast<size_t>(n));
  parallel_for(n, [&](int64_t i) {
    thread_local std::vector<double> scratch;
    Resolved& r = res[i];
    r.orig = static_cast<int32_t>(i);
    std::string m = validate(params[i], true);
    if (m.empty()) {
      MangoGpuGrid g{};
      g.kind = MANGO_GPU_GRID_AUTO;
      if (grids) g = grids[grid_stride ? i : 0];
      m = resolve(params[i], g, &r, &scratch);
    }
    if (!m.empty()) {
      r.status = MANGO_ERR_VALIDATION;
      msgs[i] = m;
    }
  });
  const double resolve_ms = ms_since(t0);
  MangoGpuBatch* b =
      create_batch_resolved(ctx, params, std::move(res), std::move(msgs), trbdf2, reuse, stream);
  b->host_prep_ms += resolve_ms;
  return b;
}

MangoGpuBatch* create_batch_resolved(MangoGpuContext* ctx, const MangoPricingParams* params,
                                     std::vector<Resolved> resolved,
                                     std::vector<std::string> messages,
                                     const MangoGpuTrbdf2* trbdf2, MangoGpuBatch* reuse,
                                     cudaStream_t stream) {
  auto t0 = Clock::now();
  const int64_t n = static_cast<int64_t>(resolved.size());
  auto keep = [](MangoGpuBatch*) {};
  std::unique_ptr<MangoGpuBatch, void (*)(MangoGpuBatch*)> b(
      reuse ? reuse : new MangoGpuBatch(), reuse ? static_cast<void (*)(MangoGpuBatch*)>(keep)
                                                 : destroy_batch);
  b->ctx = ctx;
  b->stream = stream ? stream : ctx->stream;
  b->n = n;
  b->mc = make_const(trbdf2);
  b->res = std::move(resolved);
  b->msgs = std::move(messages);
  b->msgs.resize(static_cast<size_t>(n));
  b->order.clear();
  b->ntiles = 0;
  b->algo_flops = 0;
  b->h2d_bytes = 0;
  b->host_prep_ms = 0;
  b->tv_tile0 = 0;
  b->wplan_ready = false;
  b->nwt = 0;
  b->nbins = 0;
  b->ran = false;
  b->runs = 0;
  for (auto& e : b->ev)
    if (!e) check(cudaEventCreate(&e), "cudaEventCreate");
  // Sort accepted options by n_space bucket descending (the largest tiles
  // are dequeued first and a tile's lanes have nearly the same row count),
  // then by option type (puts and calls lock at opposite ends of the grid,
  // so a mixed tile would test the lock on every row), then by n_time and
  // n_space descending and normalised moneyness ln(S/K) / (sigma sqrt(T)),
  // so that a tile's lanes meet the obstacle at similar rows and leave the
  // cached factorisation together (lanes on the off-cache path at different
  // rows serialise a warp).
  std::vector<int32_t>& order = b->order;
  struct SortKey {
    int64_t n, nt;
    double mk;
    int32_t tv, type, idx, nb;
  };
  std::vector<int32_t> valid;
  valid.reserve(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i)
    if (b->res[i].status == 0) valid.push_back(static_cast<int32_t>(i));
  const int64_t nv = static_cast<int64_t>(valid.size());
  std::vector<SortKey> keys(static_cast<size_t>(nv));
  parallel_for(nv, [&](int64_t j) {
    const int32_t i = valid[j];
    const Resolved& r = b->res[i];
    const MangoPricingParams& p = params[r.orig];
    const double k = std::log(p.spot / p.strike) / (p.volatility * std::sqrt(p.maturity));
    // n_space in buckets 4 % wide: a tile then gathers options of nearly the
    // same width, so the buckets hold enough options to keep the step
    // counts of a tile close as well.
    const int32_t nb = static_cast<int32_t>(std::floor(std::log(static_cast<double>(r.spec.n)) /
                                                       std::log(1.04)));
    keys[j] = SortKey{r.spec.n, r.nt, std::isfinite(k) ? k : 0.0, r.tv ? 1 : 0, p.option_type, i, nb};
  }, 4096);
  auto before = [](const SortKey& a, const SortKey& c) {
    if (a.tv != c.tv) return a.tv < c.tv;  // time-varying options last
    if (a.nb != c.nb) return a.nb > c.nb;
    if (a.type != c.type) return a.type < c.type;
    if (a.nt != c.nt) return a.nt > c.nt;
    if (a.n != c.n) return a.n > c.n;
    if (a.mk != c.mk) return a.mk < c.mk;
    return a.idx < c.idx;
  };
  {
    // Parallel sort: sorted runs on all host cores, then pairwise merges.
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    int64_t parts = std::min<int64_t>(hw, std::max<int64_t>(1, nv / 4096));
    std::vector<int64_t> cut(static_cast<size_t>(parts) + 1);
    for (int64_t q = 0; q <= parts; ++q) cut[q] = nv * q / parts;
    parallel_for(parts, [&](int64_t q) {
      std::sort(keys.begin() + cut[q], keys.begin() + cut[q + 1], before);
    }, 1);
    std::vector<SortKey> tmp(keys.size());
    while (parts > 1) {
      const int64_t pairs = (parts + 1) / 2;
      std::vector<int64_t> ncut(static_cast<size_t>(pairs) + 1);
      parallel_for(pairs, [&](int64_t q) {
        const int64_t a = cut[2 * q], mid = cut[std::min<int64_t>(2 * q + 1, parts)],
                      e = cut[std::min<int64_t>(2 * q + 2, parts)];
        std::merge(keys.begin() + a, keys.begin() + mid, keys.begin() + mid, keys.begin() + e,
                   tmp.begin() + a, before);
      }, 1);
      for (int64_t q = 0; q <= pairs; ++q) ncut[q] = cut[std::min<int64_t>(2 * q, parts)];
      keys.swap(tmp);
      cut.swap(ncut);
      parts = pairs;
    }
  }
  order.resize(static_cast<size_t>(nv));
  for (int64_t j = 0; j < nv; ++j) order[j] = keys[j].idx;
  const int64_t m = static_cast<int64_t>(order.size());
  const int32_t ntiles = static_cast<int32_t>((m + kTile - 1) / kTile);
  b->ntiles = ntiles;
  TileDev* tiles = static_cast<TileDev*>(b->h_tiles.get(sizeof(TileDev) * std::max(ntiles, 1)));
  int64_t off = 0, xoff = 0, foff = 0;
  double flops = 0;
  const MarchConst& mc = b->mc;
  for (int32_t t = 0; t < ntiles; ++t) {
    TileDev& td = tiles[t];
    td.first = t * kTile;
    td.count = static_cast<int32_t>(std::min<int64_t>(kTile, m - td.first));
    int64_t nx = 0, nt = 0;
    for (int l = 0; l < td.count; ++l) {
      const Resolved& r = b->res[order[td.first + l]];
      nx = std::max<int64_t>(nx, r.spec.n);
      nt = std::max<int64_t>(nt, r.nt);
      // Algorithmic FP64 work (FMA = 2): 28 per row per TR-BDF2 step, 18 per
      // row for the Rannacher start, 20 per row for the output splines; the
      // time-varying march refactors both stage matrices: 64 per row per step.
      const double steps = static_cast<double>(r.nt) - (mc.rannacher ? 1.0 : 0.0);
      flops += static_cast<double>(r.spec.n) *
               ((r.tv ? 64.0 : 28.0) * steps + (mc.rannacher ? 18.0 : 0.0) + 20.0);
    }
    td.nx = static_cast<int32_t>(nx);
    td.nt = static_cast<int32_t>(nt);
    td.off = off;
    td.xoff = xoff;
    td.foff = foff;
    off += static_cast<int64_t>(A_COUNT) * nx * kTile;
    xoff += nx * kTile;
    foff += nx * kTile;
  }
  b->algo_flops = flops;

  OptDev* opts = static_cast<OptDev*>(b->h_opts.get(sizeof(OptDev) * std::max<int64_t>(m, 1)));
  const bool dev_grids = b->device_grids;
  double* xs = dev_grids ? nullptr
                         : static_cast<double*>(b->h_xs.get(sizeof(double) * std::max<int64_t>(xoff, 1)));
  GridDev* gspec = dev_grids ? static_cast<GridDev*>(
                                   b->h_grids.get(sizeof(GridDev) * std::max<int64_t>(m, 1)))
                             : nullptr;
  // Deferred grids: the points (and the boundary data taken from them) are
  // filled later by fill_batch_grids and uploaded by upload_batch_grids.
  const bool defer = b->defer_grids && !dev_grids;
  parallel_for(ntiles, [&](int64_t t) {  // 32 grids per item: a small grain
    const TileDev& td = tiles[t];
    std::vector<double> x;
    for (int l = 0; l < kTile; ++l) {
      if (l >= td.count) {
        if (!dev_grids && !defer) {
          double* dst = xs + td.xoff + l;
          for (int i = 0; i < td.nx; ++i) dst[static_cast<size_t>(i) * kTile] = 0.0;
        }
        continue;
      }
      const Resolved& r = b->res[order[td.first + l]];
      const MangoPricingParams& p = params[r.orig];
      if (dev_grids) {
        GridDev& g = gspec[td.first + l];
        g = GridDev{};
        g.type = r.spec.type;
        g.n_clusters = r.spec.n_clusters;
        g.n = static_cast<int32_t>(r.spec.n);
        g.x_min = r.spec.x_min;
        g.x_max = r.spec.x_max;
        g.concentration = r.spec.concentration;
        for (int c = 0; c < 4; ++c) {
          g.c_center[c] = r.spec.c_center[c];
          g.c_alpha[c] = r.spec.c_alpha[c];
          g.c_weight[c] = r.spec.c_weight[c];
        }
      } else if (!defer) {
        double* dst = xs + td.xoff + l;
        x.resize(static_cast<size_t>(r.spec.n));
        generate_grid(r.spec, x.data());
        for (int i = 0; i < td.nx; ++i)
          dst[static_cast<size_t>(i) * kTile] = x[std::min<int64_t>(i, r.spec.n - 1)];
      }
      OptDev& o = opts[td.first + l];
      o.dt = (p.maturity - 0.0) / static_cast<double>(r.nt);  // TimeDomain::from_n_steps
      o.sigma = p.volatility;
      o.r = p.rate_const;
      o.q = p.dividend_yield;
      const bool put = p.option_type == MANGO_PUT;
      // american_option.cpp:192-197; with device grids, grid_finish_kernel;
      // deferred, fill_batch_grids
      o.bc_left = (dev_grids || defer) ? 0.0 : (put ? std::max(1.0 - std::exp(x[0]), 0.0) : 0.0);
      o.exp_xr = (dev_grids || defer) ? 0.0 : std::exp(x[r.spec.n - 1]);
      o.x_spot = std::log(p.spot / p.strike);
      o.spot = p.spot;
      o.strike = p.strike;
      o.n = static_cast<int32_t>(r.spec.n);
      o.nt = static_cast<int32_t>(r.nt);
      o.is_put = put ? 1 : 0;
      o.orig = r.orig;
    }
  }, 8);
  b->grids_pending = defer;
  b->grid_params = params;
  // Time-varying options: per-option data, time points, curves, events.
  int64_t nc = 0;
  while (nc < m && !b->res[order[nc]].tv) ++nc;
  // Test hook MANGO_GPU_SINGULAR_PIVOT=<caller index>: that option (when it
  // is on the constant-coefficient march) gets a zero first pivot, so its
  // slot comes back MANGO_ERR_SOLVER as after a singular Thomas solve
  // (thomas_solver.hpp:386-388).  Nothing else changes.
  b->mc.singular_pivot = -1;
  if (const char* e = std::getenv("MANGO_GPU_SINGULAR_PIVOT"))
    if (*e) {
      const long long want = std::atoll(e);
      for (int64_t k = 0; k < nc; ++k)
        if (b->res[order[k]].orig == want) b->mc.singular_pivot = static_cast<int32_t>(k);
    }
  std::vector<TvDev> tvh;
  std::vector<double> tph, curveh, evh;
  if (nc < m) {
    b->mc.tv_first = static_cast<int32_t>(nc);
    b->tv_tile0 = static_cast<int32_t>(nc / kTile);
    tvh.resize(static_cast<size_t>(m - nc));
    for (int64_t k = nc; k < m; ++k) {
      const Resolved& r = b->res[order[k]];
      const MangoPricingParams& p = params[r.orig];
      TvDev& d = tvh[static_cast<size_t>(k - nc)];
      d = TvDev{};
      d.T = p.maturity;
      d.r = p.rate_const;
      d.tp_off = -1;
      if (!r.tp.empty()) {
        d.tp_off = static_cast<int32_t>(tph.size());
        tph.insert(tph.end(), r.tp.begin(), r.tp.end());
      }
      d.curve_off = static_cast<int32_t>(curveh.size() / 2);
      if (p.n_tenor_points) {
        std::vector<MangoTenorPoint> pts(p.tenor_points, p.tenor_points + p.n_tenor_points);
        std::sort(pts.begin(), pts.end(), [](const MangoTenorPoint& a, const MangoTenorPoint& c) {
          return a.tenor < c.tenor;
        });
        for (const auto& t : pts) {
          curveh.push_back(t.tenor);
          curveh.push_back(t.log_discount);
        }
        d.n_curve = static_cast<int32_t>(pts.size());
      }
      // filter_and_merge_dividends (src/option/dividend_utils.hpp): inside
      // (0, T) with a positive amount, sorted by date, same-date amounts
      // summed; one event per dividend at tau = T - t with D/K
      // (american_option.cpp:119-144), sorted by tau.
      std::vector<MangoDividend> divs;
      for (uint64_t i = 0; i < p.n_dividends; ++i) {
        const MangoDividend& dv = p.dividends[i];
        if (dv.calendar_time > 0.0 && dv.calendar_time < p.maturity && dv.amount > 0.0)
          divs.push_back(dv);
      }
      std::sort(divs.begin(), divs.end(), [](const MangoDividend& a, const MangoDividend& c) {
        return a.calendar_time < c.calendar_time;
      });
      std::vector<MangoDividend> merged;
      for (const auto& dv : divs) {
        if (!merged.empty() && std::abs(merged.back().calendar_time - dv.calendar_time) < 1e-12)
          merged.back().amount += dv.amount;
        else
          merged.push_back(dv);
      }
      std::vector<std::pair<double, double>> ev;
      for (const auto& dv : merged) ev.emplace_back(p.maturity - dv.calendar_time, dv.amount / p.strike);
      std::sort(ev.begin(), ev.end(),
                [](const std::pair<double, double>& a, const std::pair<double, double>& c) {
                  return a.first < c.first;
                });
      d.ev_off = static_cast<int32_t>(evh.size() / 2);
      d.n_ev = static_cast<int32_t>(ev.size());
      for (const auto& e : ev) {
        evh.push_back(e.first);
        evh.push_back(e.second);
      }
    }
  }
  b->host_prep_ms = ms_since(t0);

  if (m > 0) {
    cudaStream_t st = b->stream;
    double* d_xs = static_cast<double*>(b->d_xs.get(sizeof(double) * xoff));
    OptDev* d_opts = static_cast<OptDev*>(b->d_opts.get(sizeof(OptDev) * m));
    TileDev* d_tiles = static_cast<TileDev*>(b->d_tiles.get(sizeof(TileDev) * ntiles));
    if (b->march_buffers) {
      b->d_pool.get(sizeof(double) * off);
      b->d_flags.get(static_cast<size_t>(foff));
      b->d_mode.get(sizeof(int32_t) * m);
      b->d_status.get(sizeof(int32_t) * m);
      b->d_out4.get(sizeof(double) * 4 * m);
    }
    b->d_queue.get(sizeof(int) * 4);
    check(cudaEventRecord(b->ev[0], st), "event");
    GridDev* d_grids =
        dev_grids ? static_cast<GridDev*>(b->d_grids.get(sizeof(GridDev) * m)) : nullptr;
    if (dev_grids)
      check(cudaMemcpyAsync(d_grids, gspec, sizeof(GridDev) * m, cudaMemcpyHostToDevice, st),
            "H2D grid specs");
    else if (!defer)
      check(cudaMemcpyAsync(d_xs, xs, sizeof(double) * xoff, cudaMemcpyHostToDevice, st),
            "H2D grids");
    check(cudaMemcpyAsync(d_opts, opts, sizeof(OptDev) * m, cudaMemcpyHostToDevice, st), "H2D options");
    check(cudaMemcpyAsync(d_tiles, tiles, sizeof(TileDev) * ntiles, cudaMemcpyHostToDevice, st),
          "H2D tiles");
    if (dev_grids) {
      grid_kernel<<<ntiles, 256, 0, st>>>(d_tiles, d_grids, d_xs);
      check(cudaGetLastError(), "grid_kernel launch");
      grid_finish_kernel<<<(ntiles * kTile + 127) / 128, 128, 0, st>>>(d_tiles, ntiles, d_grids,
                                                                      d_xs, d_opts);
      check(cudaGetLastError(), "grid_finish_kernel launch");
    }
    double tv_bytes = 0;
    if (!tvh.empty()) {
      auto up = [&](DevBuf& d, const void* src, size_t bytes) {
        void* dst = d.get(bytes);
        if (bytes) check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st), "H2D tv");
        tv_bytes += static_cast<double>(bytes);
      };
      up(b->d_tv, tvh.data(), sizeof(TvDev) * tvh.size());
      up(b->d_tv_tp, tph.data(), sizeof(double) * tph.size());
      up(b->d_tv_curve, curveh.data(), sizeof(double) * curveh.size());
      up(b->d_tv_ev, evh.data(), sizeof(double) * evh.size());
    }
    check(cudaEventRecord(b->ev[1], st), "event");
    b->h2d_bytes = static_cast<double>((dev_grids ? sizeof(GridDev) * m : sizeof(double) * xoff) +
                                       sizeof(OptDev) * m + sizeof(TileDev) * ntiles) +
                   tv_bytes;
  }
  return b.release();
}

void fill_batch_grids(MangoGpuBatch* b) {
  const MangoPricingParams* params = b->grid_params;
  const std::vector<int32_t>& order = b->order;
  const TileDev* tiles = b->h_tiles.as<TileDev>();
  OptDev* opts = b->h_opts.as<OptDev>();
  double* xs = b->h_xs.as<double>();
  parallel_for(b->ntiles, [&](int64_t t) {
    const TileDev& td = tiles[t];
    std::vector<double> x;
    for (int l = 0; l < kTile; ++l) {
      double* dst = xs + td.xoff + l;
      if (l >= td.count) {
        for (int i = 0; i < td.nx; ++i) dst[static_cast<size_t>(i) * kTile] = 0.0;
        continue;
      }
      const Resolved& r = b->res[order[td.first + l]];
      const MangoPricingParams& p = params[r.orig];
      x.resize(static_cast<size_t>(r.spec.n));
      generate_grid(r.spec, x.data());
      for (int i = 0; i < td.nx; ++i)
        dst[static_cast<size_t>(i) * kTile] = x[std::min<int64_t>(i, r.spec.n - 1)];
      OptDev& o = opts[td.first + l];
      const bool put = p.option_type == MANGO_PUT;
      o.bc_left = put ? std::max(1.0 - std::exp(x[0]), 0.0) : 0.0;  // american_option.cpp:192-197
      o.exp_xr = std::exp(x[r.spec.n - 1]);
    }
  }, 8);
}

void upload_batch_grids(MangoGpuBatch* b) {
  const int64_t m = static_cast<int64_t>(b->order.size());
  if (m == 0) return;
  const TileDev* tiles = b->h_tiles.as<TileDev>();
  const TileDev& tl = tiles[b->ntiles - 1];
  const int64_t xoff = tl.xoff + static_cast<int64_t>(tl.nx) * kTile;
  check(cudaMemcpyAsync(b->d_xs.p, b->h_xs.p, sizeof(double) * xoff, cudaMemcpyHostToDevice,
                        b->stream),
        "H2D grids");
  check(cudaMemcpyAsync(b->d_opts.p, b->h_opts.p, sizeof(OptDev) * m, cudaMemcpyHostToDevice,
                        b->stream),
        "H2D options");
  b->grids_pending = false;
}

namespace {

__global__ void smid_probe_kernel(int* seen, int cap) {
  unsigned smid;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
  if (threadIdx.x == 0 && smid < static_cast<unsigned>(cap)) seen[smid] = 1;
}

// The dense SM index of every %smid value, from a launch of eight blocks per
// SM; left unset (nsmid = 0) unless exactly num_sms distinct ids were seen.
void probe_sm_index(MangoGpuContext* ctx, cudaStream_t st) {
  ctx->sm_probed = true;
  constexpr int kCap = 1024;
  DevBuf d;
  int* seen = static_cast<int*>(d.get(sizeof(int) * kCap));
  check(cudaMemsetAsync(seen, 0, sizeof(int) * kCap, st), "memset smid probe");
  smid_probe_kernel<<<ctx->num_sms * 8, 32, 0, st>>>(seen, kCap);
  check(cudaGetLastError(), "smid probe launch");
  std::vector<int> h(kCap);
  check(cudaMemcpyAsync(h.data(), seen, sizeof(int) * kCap, cudaMemcpyDeviceToHost, st), "D2H");
  check(cudaStreamSynchronize(st), "stream synchronize");
  d.release();
  std::vector<int32_t> index(kCap, -1);
  int count = 0, top = 0;
  for (int i = 0; i < kCap; ++i)
    if (h[i]) {
      index[i] = count++;
      top = i + 1;
    }
  if (count != ctx->num_sms) return;
  check(cudaMemcpyAsync(ctx->d_sm_index.get(sizeof(int32_t) * top), index.data(),
                        sizeof(int32_t) * top, cudaMemcpyHostToDevice, st),
        "H2D SM index");  // pageable source: staged before the call returns
  ctx->nsmid = top;
}

}  // namespace

// Enqueue setup, march and outputs for a created batch.
void run_batch(MangoGpuBatch* b) {
  MangoGpuContext* ctx = b->ctx;
  const int64_t m = static_cast<int64_t>(b->order.size());
  b->ran = true;
  if (m == 0) return;
  cudaStream_t st = b->stream;
  const int ntiles = b->ntiles;
  const int threads = ntiles * kTile;
  const TileDev* d_tiles = b->d_tiles.as<TileDev>();
  const OptDev* d_opts = b->d_opts.as<OptDev>();
  double* d_pool = b->d_pool.as<double>();
  const double* d_xs = b->d_xs.as<double>();
  uint8_t* d_flags = b->d_flags.as<uint8_t>();
  int32_t* d_mode = b->d_mode.as<int32_t>();
  int32_t* d_status = b->d_status.as<int32_t>();
  check(cudaMemsetAsync(b->d_queue.p, 0, sizeof(int) * 4, st), "memset queue");
  const size_t slot = static_cast<size_t>(b->runs % MangoGpuBatch::kMaxTimedRuns) * 4;
  if (b->run_ev.size() < slot + 4) {
    b->run_ev.resize(slot + 4, nullptr);
    for (size_t j = slot; j < slot + 4; ++j) check(cudaEventCreate(&b->run_ev[j]), "cudaEventCreate");
  }
  ++b->runs;
  check(cudaEventRecord(b->run_ev[slot + 0], st), "event");
  check(cudaEventRecord(b->ev[2], st), "event");
  prep_kernel<<<(threads + 127) / 128, 128, 0, st>>>(d_tiles, ntiles, d_opts, d_xs, d_pool,
                                                     d_flags, d_mode, b->mc);
  check(cudaGetLastError(), "prep_kernel launch");
  check(cudaEventRecord(b->ev[3], st), "event");
  check(cudaEventRecord(b->run_ev[slot + 1], st), "event");
  if (!b->wplan_ready) {
    const int tv0 = b->mc.tv_first < m ? b->tv_tile0 : ntiles;
    const WarpPlan plan = plan_warp_tiles(b->h_tiles.as<TileDev>(), ntiles, tv0, ctx->num_sms);
    b->nwt = static_cast<int32_t>(plan.tiles.size());
    b->wR = plan.R;
    b->wblocks = plan.blocks;
    b->wconcurrent = plan.concurrent;
    if (b->nwt > 0) {
      // pageable sources: staged before the calls return
      check(cudaMemcpyAsync(b->d_wt.get(sizeof(int32_t) * b->nwt), plan.tiles.data(),
                            sizeof(int32_t) * b->nwt, cudaMemcpyHostToDevice, st),
            "H2D warp tiles");
      check(cudaMemcpyAsync(b->d_tile_warp.get(static_cast<size_t>(ntiles)), plan.flag.data(),
                            static_cast<size_t>(ntiles), cudaMemcpyHostToDevice, st),
            "H2D warp flags");
    }
    // Uneven batches (the costliest tile above 1.5x the mean; cost: rows x
    // steps of the tile's widest and longest lane): the thread march's tiles
    // go to one list per SM sub-partition, longest first to the least-loaded
    // list.  A warp's FP64 issue is shared with the other warps of its
    // sub-partition, and every warp of a 65,536-option batch holds one tile
    // for the whole launch, so which tiles share a sub-partition sets the
    // launch's length; the lists give the costliest tiles a sub-partition to
    // themselves.  MANGO_GPU_BINS=0 turns this off.
    b->nbins = 0;
    bool bins_on = true;
    if (const char* e = std::getenv("MANGO_GPU_BINS")) bins_on = std::atoi(e) != 0;
    const int nbins = 4 * ctx->num_sms;
    std::vector<int32_t> mt;
    for (int t = 0; t < tv0; ++t)
      if (b->nwt == 0 || !plan.flag[t]) mt.push_back(t);
    const TileDev* th = b->h_tiles.as<TileDev>();
    auto cost = [&](int32_t t) {
      return static_cast<double>(std::max(th[t].nx - 2, 1)) * static_cast<double>(th[t].nt);
    };
    double csum = 0.0, cmax = 0.0;
    for (int32_t t : mt) {
      csum += cost(t);
      cmax = std::max(cmax, cost(t));
    }
    const bool uneven = !mt.empty() && cmax > 1.5 * csum / static_cast<double>(mt.size());
    if (bins_on && uneven && static_cast<int64_t>(mt.size()) >= nbins) {
      if (!ctx->sm_probed) probe_sm_index(ctx, st);
      if (ctx->nsmid > 0) {
        std::stable_sort(mt.begin(), mt.end(),
                         [&](int32_t a, int32_t c) { return cost(a) > cost(c); });
        std::vector<std::vector<int32_t>> lists(static_cast<size_t>(nbins));
        using Load = std::pair<double, int>;
        std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
        for (int j = 0; j < nbins; ++j) heap.push({0.0, j});
        for (int32_t t : mt) {
          Load l = heap.top();
          heap.pop();
          lists[static_cast<size_t>(l.second)].push_back(t);
          l.first += cost(t);
          heap.push(l);
        }
        std::vector<int32_t> packed(static_cast<size_t>(nbins) + 1 + mt.size());
        int32_t off = 0;
        for (int j = 0; j < nbins; ++j) {
          packed[static_cast<size_t>(j)] = off;
          for (int32_t t : lists[static_cast<size_t>(j)])
            packed[static_cast<size_t>(nbins) + 1 + static_cast<size_t>(off++)] = t;
        }
        packed[static_cast<size_t>(nbins)] = off;
        check(cudaMemcpyAsync(b->d_bins.get(sizeof(int32_t) * packed.size()), packed.data(),
                              sizeof(int32_t) * packed.size(), cudaMemcpyHostToDevice, st),
              "H2D tile lists");  // pageable source: staged before the call returns
        b->d_bin_cnt.get(sizeof(int) * static_cast<size_t>(nbins));
        b->d_tile_done.get(static_cast<size_t>(ntiles));
        b->nbins = nbins;
      }
    }
    b->wplan_ready = true;
  }
  MarchConst mc = b->mc;
  mc.tile_warp = b->nwt > 0 ? b->d_tile_warp.as<uint8_t>() : nullptr;
  const int warps_per_block = 4;
  int bps = ctx->march_blocks_per_sm;
  // MANGO_GPU_MARCH_BLOCKS_PER_SM: resident march blocks per SM (1 to the
  // occupancy limit), for launch-shape sweeps.
  if (const char* e = std::getenv("MANGO_GPU_MARCH_BLOCKS_PER_SM")) {
    const int v = std::atoi(e);
    if (v >= 1) bps = std::min(bps, v);
  }
  const int blocks = std::max(1, std::min<int>(ctx->num_sms * bps,
                                               (ntiles + warps_per_block - 1) / warps_per_block));
  if (b->wconcurrent) {
    // the long poles on their own stream, launched first so that their
    // blocks are resident beside the persistent thread march
    if (!b->wstream) {
      check(cudaStreamCreateWithFlags(&b->wstream, cudaStreamNonBlocking), "stream");
      for (auto& e : b->wev) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    }
    check(cudaEventRecord(b->wev[0], st), "event");
    check(cudaStreamWaitEvent(b->wstream, b->wev[0], 0), "stream wait");
    wmarch_launch(b->wstream, ctx->num_sms, d_tiles, b->d_wt.as<int32_t>(), b->nwt, d_opts, d_pool,
                  d_flags, d_mode, d_status, b->d_queue.as<int>() + 1, mc, b->wR, b->wblocks);
    check(cudaEventRecord(b->wev[1], b->wstream), "event");
  }
  if (b->nwt < ntiles && b->nbins > 0) {
    // the binned launch, then one over the queue for any tile left untaken
    check(cudaMemsetAsync(b->d_bin_cnt.p, 0, sizeof(int) * static_cast<size_t>(b->nbins), st),
          "memset tile lists");
    check(cudaMemsetAsync(b->d_tile_done.p, 0, static_cast<size_t>(ntiles), st), "memset taken");
    MarchConst mb = mc;
    mb.bin_off = b->d_bins.as<int32_t>();
    mb.bin_tiles = mb.bin_off + b->nbins + 1;
    mb.bin_cnt = b->d_bin_cnt.as<int>();
    mb.sm_index = ctx->d_sm_index.as<int32_t>();
    mb.nsmid = ctx->nsmid;
    mb.nbins = b->nbins;
    mb.tile_done = b->d_tile_done.as<uint8_t>();
    // No tile hand-off here: a tile moved onto the sub-partition of one of
    // the costliest tiles, which the lists keep alone, slows the launch's
    // critical path (measured on the uneven batch: 353 -> 515 ms).
    march_kernel<<<ctx->num_sms * bps, 32 * warps_per_block, 0, st>>>(
        d_tiles, ntiles, d_opts, d_pool, d_flags, d_mode, d_status, b->d_queue.as<int>(), mb);
    check(cudaGetLastError(), "march_kernel launch");
    mc.tile_done = b->d_tile_done.as<uint8_t>();
  }
  if (b->nwt < ntiles) {
    MarchConst mh = mc;
    // tile hand-off (march.cuh) on the plain queue launch without snapshots;
    // MANGO_GPU_HANDOFF=0 turns it off
    const char* he = std::getenv("MANGO_GPU_HANDOFF");
    if (b->nbins == 0 && !mc.snap_idx && !(he && he[0] == '0')) {
      const int cap = 4 * ntiles + 1024;
      const size_t bytes = 16 + sizeof(unsigned long long) * static_cast<size_t>(cap) +
                           static_cast<size_t>(ntiles);
      char* h = static_cast<char*>(b->d_handoff.get(bytes));
      check(cudaMemsetAsync(h, 0, bytes, st), "memset hand-off");
      mh.ho_ctl = reinterpret_cast<int*>(h);
      mh.ho_slot = reinterpret_cast<unsigned long long*>(h + 16);
      mh.ho_moved = reinterpret_cast<uint8_t*>(h + 16 + sizeof(unsigned long long) * cap);
      mh.ho_cap = cap;
      mh.ho_total = ntiles;
    }
    march_kernel<<<blocks, 32 * warps_per_block, 0, st>>>(d_tiles, ntiles, d_opts, d_pool,
                                                          d_flags, d_mode, d_status,
                                                          b->d_queue.as<int>(), mh);
  }
  check(cudaGetLastError(), "march_kernel launch");
  if (b->wconcurrent)
    check(cudaStreamWaitEvent(st, b->wev[1], 0), "stream wait");
  else
    wmarch_launch(st, ctx->num_sms, d_tiles, b->d_wt.as<int32_t>(), b->nwt, d_opts, d_pool,
                  d_flags, d_mode, d_status, b->d_queue.as<int>() + 1, mc, b->wR, b->wblocks);
  if (b->mc.tv_first < m) {
    const int tv_tiles = ntiles - b->tv_tile0;
    const int tv_blocks = std::max(1, std::min<int>(ctx->num_sms * 8, (tv_tiles + 3) / 4));
    march_tv_kernel<<<tv_blocks, 128, 0, st>>>(
        d_tiles, b->tv_tile0, ntiles, d_opts, b->d_tv.as<TvDev>(), b->d_tv_tp.as<double>(),
        b->d_tv_curve.as<double>(), b->d_tv_ev.as<double>(), d_xs, d_pool, d_mode, d_status,
        b->mc);
    check(cudaGetLastError(), "march_tv_kernel launch");
  }
  check(cudaEventRecord(b->ev[4], st), "event");
  check(cudaEventRecord(b->run_ev[slot + 2], st), "event");
  outputs_kernel<<<(threads + 127) / 128, 128, 0, st>>>(d_tiles, ntiles, d_opts, d_xs, d_pool,
                                                        d_mode, d_status, b->mc,
                                                        b->d_out4.as<double>());
  check(cudaGetLastError(), "outputs_kernel launch");
  check(cudaEventRecord(b->ev[5], st), "event");
  check(cudaEventRecord(b->run_ev[slot + 3], st), "event");
}

// Wait for the batch, copy results into caller slots, update context stats.
uint64_t fetch_batch(MangoGpuBatch* b, MangoGpuAmericanOut* out, std::string* first_msg) {
  MangoGpuContext* ctx = b->ctx;
  const int64_t m = static_cast<int64_t>(b->order.size());
  Stats& S = ctx->stats;
  for (int64_t i = 0; i < b->n; ++i) {
    MangoGpuAmericanOut& o = out[i];
    o.value = o.delta = o.gamma = o.theta = NAN;
    o.status = b->res[i].status;
    o.n_space = static_cast<int32_t>(b->res[i].spec.n);
    o.n_time = static_cast<int32_t>(b->res[i].nt);
    o.reserved = 0;
    if (o.status != 0 && first_msg->empty()) *first_msg = b->msgs[i];
  }
  if (m > 0) {
    cudaStream_t st = b->stream;
    double* h_out4 = static_cast<double*>(b->h_out4.get(sizeof(double) * 4 * m));
    int32_t* h_status = static_cast<int32_t*>(b->h_status.get(sizeof(int32_t) * m));
    check(cudaMemcpyAsync(h_out4, b->d_out4.p, sizeof(double) * 4 * m, cudaMemcpyDeviceToHost, st),
          "D2H results");
    check(cudaMemcpyAsync(h_status, b->d_status.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st),
          "D2H status");
    check(cudaEventRecord(b->ev[6], st), "event");
    check(cudaStreamSynchronize(st), "stream synchronize");
    for (int64_t s = 0; s < m; ++s) {
      MangoGpuAmericanOut& o = out[b->order[s]];
      o.status = h_status[s];
      o.value = h_out4[4 * s + 0];
      o.delta = h_out4[4 * s + 1];
      o.gamma = h_out4[4 * s + 2];
      o.theta = h_out4[4 * s + 3];
    }
    float a = 0;
    if (cudaEventElapsedTime(&a, b->ev[0], b->ev[1]) == cudaSuccess) S.h2d_ms = a;
    if (cudaEventElapsedTime(&a, b->ev[2], b->ev[3]) == cudaSuccess) S.prep_ms = a;
    if (cudaEventElapsedTime(&a, b->ev[3], b->ev[4]) == cudaSuccess) S.march_ms = a;
    if (cudaEventElapsedTime(&a, b->ev[4], b->ev[5]) == cudaSuccess) S.outputs_ms = a;
    if (cudaEventElapsedTime(&a, b->ev[5], b->ev[6]) == cudaSuccess) S.d2h_ms = a;
    cudaGetLastError();  // elapsed-time queries on unrecorded events are not errors here
    S.d2h_bytes = static_cast<double>(sizeof(double) * 4 * m + sizeof(int32_t) * m);
  }
  uint64_t failed = 0;
  for (int64_t i = 0; i < b->n; ++i) failed += out[i].status != 0;
  S.options = b->n;
  S.tiles = b->ntiles;
  S.algo_flops = b->algo_flops;
  S.h2d_bytes = b->h2d_bytes;
  S.host_prep_ms = b->host_prep_ms;
  S.kernel_launches = m > 0 ? (2 + (b->nwt < b->ntiles ? 1 : 0) + (b->nwt > 0 ? 1 : 0) +
                               (b->nbins > 0 && b->nwt < b->ntiles ? 1 : 0) +
                               (b->mc.tv_first < m ? 1 : 0))
                            : 0;
  return failed;
}

}  // namespace mgpu

using namespace mgpu;

extern "C" {

const char* mango_gpu_build_info(void) {
  return "mango-option GB300 engine: sm_103a FP64 TR-BDF2/projected-Thomas march";
}

MangoStatus mango_gpu_context_create(int32_t device, MangoGpuContext** out, MangoError* err) {
  if (!out) {
    set_err(err, MANGO_ERR_VALIDATION, "out is null");
    return MANGO_ERR_VALIDATION;
  }
  *out = nullptr;
  MangoGpuContext* ctx = nullptr;
  try {
    int count = 0;
    check(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device < 0 || device >= count) throw CudaError("no such CUDA device");
    cudaDeviceProp prop{};
    check(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    if (prop.major != 10 || prop.minor != 3)
      throw CudaError("this library is built for sm_103a (GB300) only; device is sm_" +
                      std::to_string(prop.major) + std::to_string(prop.minor));
    check(cudaSetDevice(device), "cudaSetDevice");
    ctx = new MangoGpuContext();
    ctx->device = device;
    ctx->num_sms = prop.multiProcessorCount;
    check(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking), "stream");
    ctx->stream = ctx->own_stream;
    for (auto& a : ctx->aux) check(cudaStreamCreateWithFlags(&a, cudaStreamNonBlocking), "stream");
    int bps = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, march_kernel, 128, 0), "occupancy");
    ctx->march_blocks_per_sm = std::max(1, bps);
    *out = ctx;
    return MANGO_OK;
  } catch (const std::exception& e) {
    if (ctx && ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    if (ctx)
      for (auto& a : ctx->aux)
        if (a) cudaStreamDestroy(a);
    delete ctx;
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

void mango_gpu_context_destroy(MangoGpuContext* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  if (ctx->scratch) destroy_batch(ctx->scratch);
  for (int c = 0; c < 2; ++c) {
    if (ctx->aux[c]) cudaStreamSynchronize(ctx->aux[c]);
    if (ctx->chunk[c]) destroy_batch(ctx->chunk[c]);
    if (ctx->aux[c]) cudaStreamDestroy(ctx->aux[c]);
  }
  if (ctx->table_batch) destroy_batch(ctx->table_batch);
  for (auto& d : ctx->table_buf) d.release();
  for (MangoGpuBatch* ib : ctx->iv_batch)
    if (ib) destroy_batch(ib);
  for (auto& d : ctx->iv_dev) d.release();
  for (auto& h : ctx->iv_host) h.release();
  for (auto& level : ctx->iv_ws)
    for (auto& d : level) d.release();
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  ctx->d_sm_index.release();
  delete ctx;
}

MangoStatus mango_gpu_context_set_stream(MangoGpuContext* ctx, void* stream) {
  if (!ctx) return MANGO_ERR_VALIDATION;
  ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
  return MANGO_OK;
}

MangoStatus mango_gpu_batch_create(MangoGpuContext* ctx, const MangoPricingParams* params,
                                   uint64_t n, const MangoGpuGrid* grids, uint64_t grid_stride,
                                   const MangoGpuTrbdf2* trbdf2, MangoGpuBatch** out,
                                   MangoError* err) {
  if (!ctx || !out || (n > 0 && !params)) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, params or out");
    return MANGO_ERR_VALIDATION;
  }
  *out = nullptr;
  if (n > (1ull << 30)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^30 options");
    return MANGO_ERR_VALIDATION;
  }
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    *out = create_batch(ctx, params, static_cast<int64_t>(n), grids, grid_stride, trbdf2);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_batch_run(MangoGpuBatch* b, MangoError* err) {
  if (!b) {
    set_err(err, MANGO_ERR_VALIDATION, "null batch");
    return MANGO_ERR_VALIDATION;
  }
  try {
    check(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    run_batch(b);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_batch_results(MangoGpuBatch* b, MangoGpuAmericanOut* out,
                                    uint64_t* out_failed, MangoError* err) {
  if (!b || (b->n > 0 && !out)) {
    set_err(err, MANGO_ERR_VALIDATION, "null batch or out");
    return MANGO_ERR_VALIDATION;
  }
  if (!b->ran) {
    set_err(err, MANGO_ERR_VALIDATION, "mango_gpu_batch_run has not been called");
    return MANGO_ERR_VALIDATION;
  }
  try {
    check(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    std::string first;
    const uint64_t failed = fetch_batch(b, out, &first);
    if (out_failed) *out_failed = failed;
    if (failed && err) set_err(err, MANGO_OK, first.empty() ? "solver failure" : first);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_batch_value_at(MangoGpuBatch* b, const uint64_t* slots, const double* spots,
                                     uint64_t n, double* out4, MangoError* err) {
  if (!b || (n > 0 && (!slots || !spots || !out4))) {
    set_err(err, MANGO_ERR_VALIDATION, "null batch, slots, spots or out");
    return MANGO_ERR_VALIDATION;
  }
  if (!b->ran) {
    set_err(err, MANGO_ERR_VALIDATION, "mango_gpu_batch_run has not been called");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  if (n > (1ull << 30)) {
    set_err(err, MANGO_ERR_VALIDATION, "above 2^30 points");
    return MANGO_ERR_VALIDATION;
  }
  DevBuf d_grp, d_spot, d_strike, d_scratch, d_out;
  auto release = [&]() {
    for (DevBuf* d : {&d_grp, &d_spot, &d_strike, &d_scratch, &d_out}) d->release();
  };
  try {
    check(cudaSetDevice(b->ctx->device), "cudaSetDevice");
    // slot -> sorted position (-1: the slot never reached the device)
    std::vector<int32_t> pos(static_cast<size_t>(b->n), -1);
    for (size_t s = 0; s < b->order.size(); ++s) pos[b->order[s]] = static_cast<int32_t>(s);
    const OptDev* ho = b->h_opts.as<OptDev>();
    const int64_t m = static_cast<int64_t>(n);
    std::vector<int32_t> grp(static_cast<size_t>(m));
    std::vector<double> strike(static_cast<size_t>(m));
    int nmax = 3;
    for (int64_t j = 0; j < m; ++j) {
      if (slots[j] >= static_cast<uint64_t>(b->n)) {
        set_err(err, MANGO_ERR_VALIDATION, "slot out of range");
        return MANGO_ERR_VALIDATION;
      }
      const int32_t g = pos[slots[j]];
      grp[j] = g;
      strike[j] = g >= 0 ? ho[g].strike : 1.0;
      if (g >= 0) nmax = std::max(nmax, ho[g].n);
    }
    cudaStream_t st = b->stream;
    int32_t* dg = static_cast<int32_t*>(d_grp.get(sizeof(int32_t) * m));
    double* ds = static_cast<double*>(d_spot.get(sizeof(double) * m));
    double* dk = static_cast<double*>(d_strike.get(sizeof(double) * m));
    double* dscr = static_cast<double*>(d_scratch.get(sizeof(double) * 2 * nmax * m));
    double* dout = static_cast<double*>(d_out.get(sizeof(double) * 4 * m));
    check(cudaMemcpyAsync(dg, grp.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, st), "H2D");
    check(cudaMemcpyAsync(ds, spots, sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
    check(cudaMemcpyAsync(dk, strike.data(), sizeof(double) * m, cudaMemcpyHostToDevice, st), "H2D");
    chain_outputs_kernel<<<static_cast<int>((m + 127) / 128), 128, 0, st>>>(
        static_cast<int>(m), dg, ds, dk, b->d_tiles.as<TileDev>(), b->d_opts.as<OptDev>(),
        b->d_xs.as<double>(), b->d_pool.as<double>(), b->d_mode.as<int32_t>(),
        b->d_status.as<int32_t>(), b->mc, dscr, nmax, dout);
    check(cudaGetLastError(), "value_at launch");
    check(cudaMemcpyAsync(out4, dout, sizeof(double) * 4 * m, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    release();
    return MANGO_OK;
  } catch (const std::exception& e) {
    release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

void mango_gpu_batch_destroy(MangoGpuBatch* b) {
  if (!b) return;
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->stream);
  destroy_batch(b);
}

MangoStatus mango_gpu_batch_timings(MangoGpuBatch* b, int32_t reset, double* prep_ms,
                                    double* march_ms, double* outputs_ms, int64_t* runs,
                                    MangoError* err) {
  if (!b) {
    set_err(err, MANGO_ERR_VALIDATION, "null batch");
    return MANGO_ERR_VALIDATION;
  }
  try {
    check(cudaStreamSynchronize(b->stream), "stream synchronize");
    const int64_t k = std::min<int64_t>(b->runs, MangoGpuBatch::kMaxTimedRuns);
    double acc[3] = {0, 0, 0};
    for (int64_t r = 0; r < k; ++r)
      for (int j = 0; j < 3; ++j) {
        float ms = 0;
        check(cudaEventElapsedTime(&ms, b->run_ev[4 * r + j], b->run_ev[4 * r + j + 1]), "elapsed");
        acc[j] += ms;
      }
    const double d = k > 0 ? static_cast<double>(k) : 1.0;
    if (prep_ms) *prep_ms = acc[0] / d;
    if (march_ms) *march_ms = acc[1] / d;
    if (outputs_ms) *outputs_ms = acc[2] / d;
    if (runs) *runs = k;
    if (reset) b->runs = 0;
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

namespace {
// A kept batch whose device state exceeds this is freed after the call:
// the reuse saves allocation time, not worth holding a huge batch's memory.
constexpr size_t kKeepBytes = size_t(4) << 30;
void release_if_large(MangoGpuBatch*& b) {
  if (b && b->d_pool.cap > kKeepBytes) {
    destroy_batch(b);
    b = nullptr;
  }
}
}  // namespace

MangoStatus mango_gpu_price_american_batch(MangoGpuContext* ctx, const MangoPricingParams* params,
                                           uint64_t n, const MangoGpuGrid* grids,
                                           uint64_t grid_stride, const MangoGpuTrbdf2* trbdf2,
                                           MangoGpuAmericanOut* out, uint64_t* out_failed,
                                           MangoError* err) {
  if (!ctx || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, params or out");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 30)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^30 options");
    return MANGO_ERR_VALIDATION;
  }
  auto t0 = Clock::now();
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int64_t nn = static_cast<int64_t>(n);
    // Large batches: k chunks alternating over two streams and two reused
    // batches; chunk c is prepared on the host while chunk c-1 runs, and
    // chunk c-2's results are collected before its buffers are refilled.
    // Chunks keep at least kChunkMin options, so each march still has
    // several tiles per resident warp (a smaller chunk cannot fill the GPU).
    constexpr int64_t kChunkMin = 32768;
    const int k = static_cast<int>(std::min<int64_t>(4, std::max<int64_t>(1, nn / kChunkMin)));
    if (k > 1) {
      cudaEvent_t start = nullptr;
      check(cudaEventCreateWithFlags(&start, cudaEventDisableTiming), "event");
      check(cudaEventRecord(start, ctx->stream), "event");
      for (auto a : ctx->aux) {
        check(cudaStreamSynchronize(a), "stream synchronize");
        check(cudaStreamWaitEvent(a, start, 0), "stream wait");
      }
      cudaEventDestroy(start);
      Stats acc{};
      uint64_t failed = 0;
      std::string first;
      std::vector<int64_t> off(static_cast<size_t>(k) + 1);
      for (int c = 0; c <= k; ++c) off[c] = nn * c / k;
      auto collect = [&](int c) {
        failed += fetch_batch(ctx->chunk[c % 2], out + off[c], &first);
        const Stats& S = ctx->stats;
        acc.host_prep_ms += S.host_prep_ms;
        acc.h2d_ms += S.h2d_ms;
        acc.prep_ms += S.prep_ms;
        acc.march_ms += S.march_ms;
        acc.outputs_ms += S.outputs_ms;
        acc.d2h_ms += S.d2h_ms;
        acc.options += S.options;
        acc.tiles += S.tiles;
        acc.kernel_launches += S.kernel_launches;
        acc.algo_flops += S.algo_flops;
        acc.h2d_bytes += S.h2d_bytes;
        acc.d2h_bytes += S.d2h_bytes;
      };
      for (int c = 0; c < k; ++c) {
        if (c >= 2) collect(c - 2);
        const MangoGpuGrid* g = grids ? grids + (grid_stride ? off[c] : 0) : nullptr;
        ctx->chunk[c % 2] = create_batch(ctx, params + off[c], off[c + 1] - off[c], g, grid_stride,
                                         trbdf2, ctx->chunk[c % 2], ctx->aux[c % 2]);
        run_batch(ctx->chunk[c % 2]);
      }
      for (int c = std::max(0, k - 2); c < k; ++c) collect(c);
      for (auto& cb : ctx->chunk) release_if_large(cb);
      acc.total_ms = ms_since(t0);
      ctx->stats = acc;
      if (out_failed) *out_failed = failed;
      if (failed && err) set_err(err, MANGO_OK, first.empty() ? "solver failure" : first);
      return MANGO_OK;
    }
    // The context's scratch batch: its device and pinned host buffers are
    // reused (grow-only) by the next call, once no copy of an earlier call
    // (one that failed midway) can still touch them.
    if (ctx->scratch) check(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    MangoGpuBatch* b = create_batch(ctx, params, static_cast<int64_t>(n), grids, grid_stride,
                                    trbdf2, ctx->scratch);
    ctx->scratch = b;
    run_batch(b);
    std::string first;
    const uint64_t failed = fetch_batch(b, out, &first);
    release_if_large(ctx->scratch);
    if (out_failed) *out_failed = failed;
    if (failed && err) set_err(err, MANGO_OK, first.empty() ? "solver failure" : first);
    ctx->stats.total_ms = ms_since(t0);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_fp64_probe(MangoGpuContext* ctx, double* tflops, MangoError* err) {
  if (!ctx || !tflops) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const int blocks = ctx->num_sms * 8, threads = 256, iters = 2048;
    double* d = nullptr;
    check(cudaMallocAsync(reinterpret_cast<void**>(&d), sizeof(double) * blocks * threads, st),
          "cudaMallocAsync");
    cudaEvent_t e0, e1;
    check(cudaEventCreate(&e0), "event");
    check(cudaEventCreate(&e1), "event");
    fp64_probe_kernel<<<blocks, threads, 0, st>>>(d, 64);  // warm-up
    double best = 0;
    for (int rep = 0; rep < 3; ++rep) {
      check(cudaEventRecord(e0, st), "event");
      fp64_probe_kernel<<<blocks, threads, 0, st>>>(d, iters);
      check(cudaEventRecord(e1, st), "event");
      check(cudaEventSynchronize(e1), "event sync");
      float ms = 0;
      check(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
      // 16 independent chains x iters FMAs per thread, 2 flops each
      const double fl = 2.0 * 16.0 * iters * static_cast<double>(blocks) * threads;
      best = std::max(best, fl / (ms * 1e-3) / 1e12);
    }
    check(cudaFreeAsync(d, st), "cudaFreeAsync");
    check(cudaStreamSynchronize(st), "sync");
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_resolve_grid(const MangoPricingParams* params, const MangoGpuGrid* grid,
                                   double* x_out, int64_t cap, int64_t* n_space,
                                   int64_t* n_time, MangoError* err) {
  if (!params || !n_space || !n_time) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  try {
    std::string m = validate(*params, true);
    Resolved r;
    std::vector<double> scratch;
    if (m.empty()) {
      MangoGpuGrid g{};
      g.kind = MANGO_GPU_GRID_AUTO;
      if (grid) g = *grid;
      m = resolve(*params, g, &r, &scratch);
    }
    if (!m.empty()) {
      set_err(err, MANGO_ERR_VALIDATION, m);
      return MANGO_ERR_VALIDATION;
    }
    *n_space = r.spec.n;
    *n_time = r.nt;
    if (x_out && cap >= r.spec.n) generate_grid(r.spec, x_out);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_last_stats(const MangoGpuContext* ctx, MangoGpuStats* out) {
  if (!ctx || !out) return MANGO_ERR_VALIDATION;
  const Stats& s = ctx->stats;
  out->host_prep_ms = s.host_prep_ms;
  out->h2d_ms = s.h2d_ms;
  out->prep_ms = s.prep_ms;
  out->march_ms = s.march_ms;
  out->outputs_ms = s.outputs_ms;
  out->d2h_ms = s.d2h_ms;
  out->total_ms = s.total_ms;
  out->algo_flops = s.algo_flops;
  out->h2d_bytes = s.h2d_bytes;
  out->d2h_bytes = s.d2h_bytes;
  out->options = s.options;
  out->tiles = s.tiles;
  out->kernel_launches = s.kernel_launches;
  for (int j = 0; j < 2; ++j) out->iv_evals[j] = s.iv_evals[j];
  return MANGO_OK;
}

}  // extern "C"
