// table.cu -- price-table PDE sweep on the GPU.
//
// Restates PriceTableBuilderND<4>::make_batch, solve_batch and
// extract_tensor (src/option/table/bspline/bspline_builder.cpp:198-480):
// one American option per (sigma, r) pair at S = K = K_ref and T = max tau,
// marched with snapshot taps at the maturity axis, then each snapshot
// resampled onto the log-moneyness axis with a natural cubic spline.  The
// grid routing (shared auto grid, explicit grid, or the per-slice fallback
// through the normalized-chain path of BatchAmericanOptionSolver) is
// decided on the host exactly as the reference decides it; the GPU runs the
// marches (one persistent launch for all slices) and the resampling.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"

namespace mgpu {

namespace {

// BatchAmericanOptionSolver limits (src/option/american_option_batch.hpp:219-221).
constexpr double kMaxWidth = 5.8;
constexpr double kMaxDx = 0.05;
constexpr double kMinMarginAbs = 0.35;

struct SliceParam {
  double sigma, r;
};

// estimate_batch_pde_grid (src/option/grid_spec_types.cpp:120-177) for
// options with spot = strike and maturity T.
void estimate_batch(const std::vector<SliceParam>& ps, double T, const Accuracy& acc,
                    GridSpec* spec, int64_t* nt) {
  double gmin = 1e300, gmax = -1e300;
  int64_t gnx = 0, gnt = 0;
  std::vector<double> scratch;
  for (const auto& p : ps) {
    GridSpec s;
    int64_t n_t = 0;
    estimate_grid(1.0, 1.0, T, p.sigma, acc, &s, &n_t, &scratch);
    gmin = std::min(gmin, s.x_min);
    gmax = std::max(gmax, s.x_max);
    gnx = std::max<int64_t>(gnx, s.n);
    gnt = std::max<int64_t>(gnt, n_t);
  }
  GridSpec s;
  s.n = gnx;
  s.x_min = gmin;
  s.x_max = gmax;
  const bool ok = gnx >= 2 && gmin < gmax && 0.0 >= gmin && 0.0 <= gmax && acc.alpha > 0;
  if (ok) {
    s.type = GridSpec::MultiSinh;
    s.n_clusters = 1;
    s.c_center[0] = 0.0;
    s.c_alpha[0] = acc.alpha;
    s.c_weight[0] = 1.0;
  } else {
    s = sinh_spec(gmin, gmax, gnx, acc.alpha);
  }
  *spec = s;
  *nt = gnt;
}

// ensure_moneyness_coverage (bspline_builder.cpp:233-255).
void ensure_coverage(Accuracy* acc, const std::vector<SliceParam>& ps, double T, double m_lo,
                     double m_hi) {
  const double half = std::max(std::fabs(m_lo), std::fabs(m_hi));
  double mx = 0.0;
  for (const auto& p : ps) mx = std::max(mx, p.sigma * std::sqrt(T));
  mx = std::max(mx, 1e-10);
  acc->n_sigma = std::max(acc->n_sigma, (half / mx) * 1.1);
}

// BatchAmericanOptionSolver::is_normalized_eligible for a table batch
// (american_option_batch.cpp:26-107): one option type, no dividends, all
// moneyness 1, so only the grid checks on the first option remain.
bool normalized_eligible(const SliceParam& first, double T, const Accuracy& acc) {
  GridSpec s;
  int64_t n_t = 0;
  std::vector<double> scratch;
  estimate_grid(1.0, 1.0, T, first.sigma, acc, &s, &n_t, &scratch);
  const double dx = (s.x_max - s.x_min) / static_cast<double>(s.n - 1);
  if (dx > kMaxDx) return false;
  if (s.x_max - s.x_min > kMaxWidth) return false;
  const double margin_left = 0.0 - s.x_min, margin_right = s.x_max - 0.0;
  const double min_margin = std::max(kMinMarginAbs, 6.0 * dx);
  return !(margin_left < min_margin || margin_right < min_margin);
}

}  // namespace

// Snapshot kernels --------------------------------------------------------

// One thread per (slice, snapshot): natural cubic spline through the
// snapshot (CubicSpline::build, cubic_spline_solver.hpp:74-170) evaluated at
// every moneyness point (eval, :176-189) into tensor[m][tau][sigma][r].
__global__ void resample_kernel(int nslices, int ntau, int nm, int ns, int nr,
                                const int32_t* __restrict__ slice_k, const OptDev* __restrict__ opts,
                                const double* __restrict__ xs, const TileDev* __restrict__ tiles,
                                const int32_t* __restrict__ status,
                                const int32_t* __restrict__ snap_count,
                                const int64_t* __restrict__ snap_off,
                                const double* __restrict__ snaps, const double* __restrict__ mgrid,
                                double* __restrict__ scratch, int64_t scratch_stride,
                                double* __restrict__ tensor) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nslices * ntau) return;
  const int s = tid / ntau, j = tid % ntau;
  const int sig_i = s / nr, r_i = s % nr;
  auto out = [&](int i) -> double& {
    return tensor[((static_cast<size_t>(i) * ntau + j) * ns + sig_i) * nr + r_i];
  };
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const int k = slice_k[s];
  if (k < 0 || status[k] != kStatusOk || j >= snap_count[k]) {
    for (int i = 0; i < nm; ++i) out(i) = nan;
    return;
  }
  const OptDev o = opts[k];
  const int n = o.n;
  const TileDev td = tiles[k / kTile];
  const double* X = xs + td.xoff + (k % kTile);
  auto x = [&](int i) { return X[static_cast<size_t>(i) * kTile]; };
  const double* y = snaps + snap_off[k] + static_cast<size_t>(j) * n;
  double* c = scratch + static_cast<size_t>(tid) * scratch_stride;  // n values
  double* cp = c + n;                                                 // n values
  double* dp = cp + n;                                                // n values
  auto h = [&](int i) { return x(i + 1) - x(i); };
  c[0] = 0.0;
  c[n - 1] = 0.0;
  const int m = n - 2;
  if (m == 1) {
    const double sr = (y[2] - y[1]) / h(1), sl = (y[1] - y[0]) / h(0);
    c[1] = (3.0 * (sr - sl)) / (2.0 * (h(0) + h(1)));
  } else if (m >= 2) {
    auto rhs = [&](int q) {
      const double sr = (y[q + 2] - y[q + 1]) / h(q + 1);
      const double sl = (y[q + 1] - y[q]) / h(q);
      return 3.0 * (sr - sl);
    };
    const double d0 = 2.0 * (h(0) + h(1));
    cp[0] = h(1) / d0;
    dp[0] = rhs(0) / d0;
    for (int q = 1; q < m - 1; ++q) {
      const double denom = fma(-h(q), cp[q - 1], 2.0 * (h(q) + h(q + 1)));
      const double inv = 1.0 / denom;
      cp[q] = h(q + 1) * inv;
      dp[q] = fma(-h(q), dp[q - 1], rhs(q)) * inv;
    }
    {
      const int q = m - 1;
      const double denom = fma(-h(q), cp[q - 1], 2.0 * (h(q) + h(q + 1)));
      dp[q] = fma(-h(q), dp[q - 1], rhs(q)) / denom;
    }
    double sol = dp[m - 1];
    c[m] = sol;
    for (int q = m - 1; q > 0; --q) {
      sol = fma(-cp[q - 1], sol, dp[q - 1]);
      c[q] = sol;
    }
  }
  for (int i = 0; i < nm; ++i) {
    const double xe = mgrid[i];
    int iv;
    if (xe <= x(0)) {
      iv = 0;
    } else if (xe >= x(n - 1)) {
      iv = n - 2;
    } else {
      int lo = 0, hi = n;
      while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (x(mid) < xe) lo = mid + 1; else hi = mid;
      }
      iv = lo;
      if (iv > 0 && (iv == n || x(iv) > xe)) --iv;
      iv = iv < n - 2 ? iv : n - 2;
    }
    const double hv = h(iv);
    const double b = (y[iv + 1] - y[iv]) / hv - hv * (2.0 * c[iv] + c[iv + 1]) / 3.0;
    const double d = (c[iv + 1] - c[iv]) / (3.0 * hv);
    const double dx = xe - x(iv);
    out(i) = y[iv] + b * dx + c[iv] * (dx * dx) + d * (dx * dx * dx);
  }
}

// Argument checks of the sweep (PriceTableBuilderND<4>::from_vectors and
// make_batch preconditions, bspline_builder.cpp:198-226, 533-620); empty
// string when the arguments are accepted.
std::string check_table_args(const double* moneyness, uint64_t nm, const double* maturity,
                             uint64_t ntau, const double* volatility, uint64_t nsig,
                             const double* rate, uint64_t nr, double K_ref, double dividend_yield,
                             MangoOptionType option_type) {
  if (!moneyness || !maturity || !volatility || !rate) return "null axis";
  if (nm < 1 || ntau < 1 || nsig < 1 || nr < 1 || nsig * nr > (1u << 24))
    return "empty or oversized axis";
  if (!(K_ref > 0.0) || dividend_yield < 0.0 ||
      (option_type != MANGO_PUT && option_type != MANGO_CALL))
    return "invalid K_ref, dividend yield or option type";
  for (uint64_t i = 1; i < ntau; ++i)
    if (!(maturity[i] > maturity[i - 1])) return "maturity axis must be strictly increasing";
  return {};
}

// The sweep with the tensor left on the device (dten: nm*ntau*nsig*nr
// doubles, [m][tau][sigma][r], NaN for failed slices).  Returns the number of
// failed slices; throws on a CUDA or argument error.
uint64_t table_sweep_device(MangoGpuContext* ctx, const double* moneyness, uint64_t nm,
                            const double* maturity, uint64_t ntau, const double* volatility,
                            uint64_t nsig, const double* rate, uint64_t nr, double K_ref,
                            double dividend_yield, MangoOptionType option_type,
                            const MangoGpuGrid* grid, double* dten, int64_t* slice_dims) {
  // The batch is the context's, refilled call after call; an exception
  // leaves it in an unknown state, so it is dropped then.
  MangoGpuBatch* b = nullptr;
  struct Guard {
    MangoGpuContext* ctx;
    MangoGpuBatch** b;
    bool ok = false;
    ~Guard() {
      if (ok || !*b) return;
      destroy_batch(*b);
      if (ctx->table_batch == *b) ctx->table_batch = nullptr;
    }
  } guard{ctx, &b};
  {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    const double T = maturity[ntau - 1];
    // make_batch: (sigma, r) cartesian product, sigma outer (bspline_builder.cpp:214-226).
    const int64_t ns = static_cast<int64_t>(nsig * nr);
    std::vector<SliceParam> ps(static_cast<size_t>(ns));
    std::vector<MangoPricingParams> pp(static_cast<size_t>(ns));
    for (uint64_t a = 0; a < nsig; ++a)
      for (uint64_t c = 0; c < nr; ++c) {
        const size_t s = a * nr + c;
        ps[s] = {volatility[a], rate[c]};
        MangoPricingParams& p = pp[s];
        std::memset(&p, 0, sizeof(p));
        p.spot = K_ref;
        p.strike = K_ref;
        p.maturity = T;
        p.volatility = volatility[a];
        p.rate_const = rate[c];
        p.dividend_yield = dividend_yield;
        p.option_type = option_type;
      }
    // solve_batch grid routing (bspline_builder.cpp:278-372).
    std::vector<GridSpec> spec(static_cast<size_t>(ns));
    std::vector<int64_t> nts(static_cast<size_t>(ns));
    const Accuracy def = default_accuracy();
    auto share = [&](const GridSpec& g, int64_t nt) {
      for (int64_t s = 0; s < ns; ++s) {
        spec[s] = g;
        nts[s] = nt;
      }
    };
    double max_sst = 0.0;
    for (const auto& p : ps) max_sst = std::max(max_sst, p.sigma * std::sqrt(T));
    if (!grid || grid->kind == MANGO_GPU_GRID_AUTO) {
      Accuracy acc = def;
      ensure_coverage(&acc, ps, T, moneyness[0], moneyness[nm - 1]);
      GridSpec g;
      int64_t nt = 0;
      estimate_batch(ps, T, acc, &g, &nt);
      share(g, nt);
    } else if (grid->kind == MANGO_GPU_GRID_SINH || grid->kind == MANGO_GPU_GRID_UNIFORM) {
      const bool sinh = grid->kind == MANGO_GPU_GRID_SINH;
      if (grid->n_space < 3 || grid->n_time < 1 || !(grid->x_min < grid->x_max) ||
          (sinh && !(grid->alpha > 0.0)))
        throw std::invalid_argument("invalid explicit table grid");
      const GridSpec ge = sinh ? sinh_spec(grid->x_min, grid->x_max, grid->n_space, grid->alpha)
                               : uniform_spec(grid->x_min, grid->x_max, grid->n_space);
      const double width = ge.x_max - ge.x_min;
      double max_dx;
      if (!sinh) {
        max_dx = width / static_cast<double>(ge.n - 1);
      } else {
        std::vector<double> xg(static_cast<size_t>(ge.n));
        generate_grid(ge, xg.data());
        max_dx = xg[1] - xg[0];
        for (int64_t i = 2; i < ge.n; ++i) max_dx = std::max(max_dx, xg[i] - xg[i - 1]);
      }
      if (width <= kMaxWidth && max_dx <= kMaxDx && width >= 6.0 * max_sst) {
        share(ge, grid->n_time);
      } else {
        // Fallback: auto estimation pinned to the requested size.
        Accuracy acc = def;
        const int64_t clamped = std::clamp<int64_t>(ge.n, 100, 1200);
        acc.min_points = acc.max_points = clamped;
        acc.max_steps = grid->n_time;
        if (sinh) acc.alpha = ge.concentration;
        const double max_abs_x = std::max(std::fabs(ge.x_min), std::fabs(ge.x_max));
        acc.n_sigma = std::max(5.0, (max_abs_x / std::max(max_sst, 1e-10)) * 1.1);
        ensure_coverage(&acc, ps, T, moneyness[0], moneyness[nm - 1]);
        if (normalized_eligible(ps[0], T, acc)) {
          // solve_normalized_chain: one S = K = 1 solve per slice on its own
          // estimate_batch_pde_grid (american_option_batch.cpp:313-382).
          parallel_for(ns, [&](int64_t s) {
            std::vector<SliceParam> one{ps[s]};
            estimate_batch(one, T, acc, &spec[s], &nts[s]);
          });
        } else {
          GridSpec g;
          int64_t nt = 0;
          estimate_batch(ps, T, acc, &g, &nt);
          share(g, nt);
        }
      }
    } else {
      throw std::invalid_argument("table grid must be AUTO, SINH or UNIFORM");
    }

    std::vector<Resolved> res(static_cast<size_t>(ns));
    for (int64_t s = 0; s < ns; ++s) {
      res[s].spec = spec[s];
      res[s].nt = nts[s];
      res[s].orig = static_cast<int32_t>(s);
      if (spec[s].n < 3 || nts[s] < 1) res[s].status = MANGO_ERR_VALIDATION;
    }
    b = create_batch_resolved(ctx, pp.data(), std::move(res),
                              std::vector<std::string>(static_cast<size_t>(ns)), nullptr,
                              ctx->table_batch);
    ctx->table_batch = b;
    const int64_t m = static_cast<int64_t>(b->order.size());
    // Snapshot indices per slice: convert_times_to_indices (grid.hpp:627-700),
    // uniform time points, sorted and de-duplicated.
    std::vector<int32_t> slice_k(static_cast<size_t>(ns), -1);
    std::vector<int32_t> sbegin(static_cast<size_t>(std::max<int64_t>(m, 1)));
    std::vector<int32_t> scount(static_cast<size_t>(std::max<int64_t>(m, 1)));
    std::vector<int64_t> soff(static_cast<size_t>(std::max<int64_t>(m, 1)));
    std::vector<int32_t> sidx;
    int64_t snap_total = 0;
    int32_t max_n = 3;
    for (int64_t k = 0; k < m; ++k) {
      const int32_t s = b->order[k];
      slice_k[s] = static_cast<int32_t>(k);
      const Resolved& r = b->res[s];
      const double dt = T / static_cast<double>(r.nt);
      std::vector<int32_t> idx;
      for (uint64_t j = 0; j < ntau; ++j) {
        int64_t st = static_cast<int64_t>(std::floor((maturity[j] - 0.0) / dt + 0.5));
        st = std::min<int64_t>(st, r.nt);
        idx.push_back(static_cast<int32_t>(st));
      }
      std::sort(idx.begin(), idx.end());
      idx.erase(std::unique(idx.begin(), idx.end()), idx.end());
      sbegin[k] = static_cast<int32_t>(sidx.size());
      scount[k] = static_cast<int32_t>(idx.size());
      soff[k] = snap_total;
      snap_total += static_cast<int64_t>(idx.size()) * r.spec.n;
      sidx.insert(sidx.end(), idx.begin(), idx.end());
      max_n = std::max<int32_t>(max_n, static_cast<int32_t>(r.spec.n));
    }
    uint64_t failed = 0;
    if (m > 0) {
      cudaStream_t st = ctx->stream;
      DevBuf& d_sidx = ctx->table_buf[0];
      DevBuf& d_sbegin = ctx->table_buf[1];
      DevBuf& d_scount = ctx->table_buf[2];
      DevBuf& d_soff = ctx->table_buf[3];
      DevBuf& d_snaps = ctx->table_buf[4];
      DevBuf& d_slice = ctx->table_buf[5];
      DevBuf& d_m = ctx->table_buf[6];
      DevBuf& d_scratch = ctx->table_buf[7];
      int32_t* dsidx = static_cast<int32_t*>(d_sidx.get(sizeof(int32_t) * std::max<size_t>(sidx.size(), 1)));
      int32_t* dsb = static_cast<int32_t*>(d_sbegin.get(sizeof(int32_t) * m));
      int32_t* dsc = static_cast<int32_t*>(d_scount.get(sizeof(int32_t) * m));
      int64_t* dso = static_cast<int64_t*>(d_soff.get(sizeof(int64_t) * m));
      double* dsnap = static_cast<double*>(d_snaps.get(sizeof(double) * std::max<int64_t>(snap_total, 1)));
      int32_t* dslice = static_cast<int32_t*>(d_slice.get(sizeof(int32_t) * ns));
      double* dm = static_cast<double*>(d_m.get(sizeof(double) * nm));
      const int64_t work = ns * static_cast<int64_t>(ntau);
      const int64_t stride = 3 * static_cast<int64_t>(max_n);
      double* dscr = static_cast<double*>(d_scratch.get(sizeof(double) * stride * work));
      check(cudaMemcpyAsync(dsidx, sidx.data(), sizeof(int32_t) * sidx.size(), cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dsb, sbegin.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dsc, scount.data(), sizeof(int32_t) * m, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dso, soff.data(), sizeof(int64_t) * m, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dslice, slice_k.data(), sizeof(int32_t) * ns, cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dm, moneyness, sizeof(double) * nm, cudaMemcpyHostToDevice, st), "H2D");
      b->mc.snap_idx = dsidx;
      b->mc.snap_begin = dsb;
      b->mc.snap_count = dsc;
      b->mc.snap_off = dso;
      b->mc.snap_out = dsnap;
      b->mc.value_only = 1;
      run_batch(b);
      const int tb = 128;
      resample_kernel<<<static_cast<int>((work + tb - 1) / tb), tb, 0, st>>>(
          static_cast<int>(ns), static_cast<int>(ntau), static_cast<int>(nm),
          static_cast<int>(nsig), static_cast<int>(nr), dslice, b->d_opts.as<OptDev>(),
          b->d_xs.as<double>(), b->d_tiles.as<TileDev>(), b->d_status.as<int32_t>(), dsc, dso,
          dsnap, dm, dscr, stride, dten);
      check(cudaGetLastError(), "resample_kernel launch");
      std::vector<int32_t> hst(static_cast<size_t>(m));
      check(cudaMemcpyAsync(hst.data(), b->d_status.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st), "D2H");
      check(cudaEventRecord(b->ev[6], st), "event");
      check(cudaStreamSynchronize(st), "stream synchronize");
      for (int64_t k = 0; k < m; ++k) failed += hst[k] != kStatusOk;
      // the call's stats: host preparation, setup, march (with snapshots),
      // then the value-only outputs and the resampling together
      Stats& S = ctx->stats;
      S = Stats{};
      float a = 0;
      S.host_prep_ms = b->host_prep_ms;
      if (cudaEventElapsedTime(&a, b->ev[2], b->ev[3]) == cudaSuccess) S.prep_ms = a;
      if (cudaEventElapsedTime(&a, b->ev[3], b->ev[4]) == cudaSuccess) S.march_ms = a;
      if (cudaEventElapsedTime(&a, b->ev[4], b->ev[6]) == cudaSuccess) S.outputs_ms = a;
      cudaGetLastError();
      S.options = m;
      S.tiles = b->ntiles;
    }
    if (m == 0)  // no slice reached the device: every tensor entry is NaN
      check(cudaMemsetAsync(dten, 0xFF, sizeof(double) * nm * ntau * nsig * nr, ctx->stream),
            "memset tensor");
    failed += static_cast<uint64_t>(ns - m);
    if (slice_dims)
      for (int64_t s = 0; s < ns; ++s) {
        slice_dims[2 * s] = b->res[s].status == 0 ? b->res[s].spec.n : -1;
        slice_dims[2 * s + 1] = b->res[s].status == 0 ? b->res[s].nt : -1;
      }
    guard.ok = true;
    return failed;
  }
}

}  // namespace mgpu

using namespace mgpu;

extern "C" MangoStatus mango_gpu_price_table_sweep(
    MangoGpuContext* ctx, const double* moneyness, uint64_t nm, const double* maturity,
    uint64_t ntau, const double* volatility, uint64_t nsig, const double* rate, uint64_t nr,
    double K_ref, double dividend_yield, MangoOptionType option_type, const MangoGpuGrid* grid,
    double* tensor, int64_t* slice_dims, uint64_t* out_failed_slices, MangoError* err) {
  const std::string bad = check_table_args(moneyness, nm, maturity, ntau, volatility, nsig, rate,
                                           nr, K_ref, dividend_yield, option_type);
  if (!ctx || !tensor || !bad.empty()) {
    set_err(err, MANGO_ERR_VALIDATION, bad.empty() ? "null argument" : bad);
    return MANGO_ERR_VALIDATION;
  }
  DevBuf d_tensor;
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    const size_t tensor_n = nm * ntau * nsig * nr;
    double* dten = static_cast<double*>(d_tensor.get(sizeof(double) * tensor_n));
    const uint64_t failed =
        table_sweep_device(ctx, moneyness, nm, maturity, ntau, volatility, nsig, rate, nr, K_ref,
                           dividend_yield, option_type, grid, dten, slice_dims);
    check(cudaMemcpyAsync(tensor, dten, sizeof(double) * tensor_n, cudaMemcpyDeviceToHost,
                          ctx->stream),
          "D2H tensor");
    check(cudaStreamSynchronize(ctx->stream), "stream synchronize");
    d_tensor.release();
    if (out_failed_slices) *out_failed_slices = failed;
    return MANGO_OK;
  } catch (const std::exception& e) {
    d_tensor.release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}
