// surface.cu -- price-table surface on the GPU: separable collocation fit,
// EEP decomposition, the assembled table and its batched price query.
//
// Restates, for the 4D standard table:
//   BSplineNDSeparable<double,4>::fit (src/math/bspline/bspline_nd_separable.hpp:153-384)
//     with BSplineCollocation1D::fit_with_workspace
//     (src/math/bspline/bspline_collocation.hpp:326-390): axes in the order
//     3, 2, 1, 0; per slice along the axis, solve B c = f, residual
//     max |B c - f| (fma order of compute_residual_from_span), a slice whose
//     residual exceeds the tolerance keeps its input values and counts as
//     failed;
//   eep_decompose with AnalyticalEEP over BSplineTensorAccessor
//     (src/option/table/eep/eep_decomposer.hpp:14-80,
//     src/option/table/bspline/bspline_tensor_accessor.hpp:16-56): the tensor
//     entry becomes eep_floor(K_ref V - European(K_ref e^m, K_ref, tau, sigma, r));
//   PriceTableBuilderND<4>::build steps 3-5
//     (src/option/table/bspline/bspline_builder.cpp:140-196) and
//     make_bspline_surface (src/option/table/bspline/bspline_surface.cpp:9-37);
//   the query AnyPriceTable::price -> EEPLayer::price -> TransformLeaf::price
//     (src/option/price_table_factory.cpp:746-751,
//     src/option/table/eep/eep_layer.hpp:21-25,
//     src/option/table/transform_leaf.hpp:28-33) with StandardTransform4D
//     coordinates (log(S/K), tau, sigma, r) and the closed-form European
//     price of EuropeanOptionResult::compute_price
//     (src/option/european_option.cpp:25-51).
//
// GB300 design: the collocation factors of an axis are computed once on the
// host (fit_host.cpp) and broadcast through shared memory; one thread solves
// one slice in place, ping-ponging between two device tensors, so a whole
// table build (sweep -> EEP -> fit -> surface) never leaves the device.
#include <cuda_runtime.h>

#include <cstdlib>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "brent.cuh"
#include "bspline.cuh"
#include "fit_host.hpp"

namespace mgpu {

MangoGpuBSpline4D* new_surface(MangoGpuContext* ctx, const double* grids, const int64_t* sizes);

namespace {

__device__ __forceinline__ double norm_cdf(double x) {
  return 0.5 * erfc(-x * 0.70710678118654752440);  // european_option.hpp:30-32
}

// EuropeanOptionResult::compute_price (european_option.cpp:25-51).
__device__ double european_price(double S, double K, double tau, double sigma, double r, double q,
                                 bool put) {
  if (tau <= 0.0 || sigma <= 0.0) {
    double s = S, k = K;
    if (tau > 0.0) {
      s = S * exp(-q * tau);
      k = K * exp(-r * tau);
    }
    return put ? fmax(k - s, 0.0) : fmax(s - k, 0.0);
  }
  const double sst = sigma * sqrt(tau);
  const double d1 = (log(S / K) + (r - q + 0.5 * sigma * sigma) * tau) / sst;
  const double d2 = d1 - sigma * sqrt(tau);
  const double eq = exp(-q * tau), er = exp(-r * tau);
  if (put) return K * er * norm_cdf(-d2) - S * eq * norm_cdf(-d1);
  return S * eq * norm_cdf(d1) - K * er * norm_cdf(d2);
}

// bs_vega (european_option.hpp:43-48), EuropeanOptionResult::vega.
__device__ double european_vega(double S, double K, double tau, double sigma, double r, double q) {
  const double d1 = (log(S / K) + (r - q + 0.5 * sigma * sigma) * tau) / (sigma * sqrt(tau));
  return S * exp(-q * tau) * sqrt(tau) * (0.3989422804014327 * exp(-0.5 * d1 * d1));
}

__device__ __forceinline__ double norm_pdf(double x) {
  return 0.3989422804014327 * exp(-0.5 * x * x);  // european_option.hpp:24-27
}

// EuropeanOptionResult::delta/gamma/theta/rho (european_option.cpp:55-154)
// with d1 = bs_d1, d2 = d1 - sigma sqrt(tau); g = {delta, gamma, theta, rho}.
__device__ void european_greeks(double S, double K, double tau, double sigma, double r, double q,
                                bool put, double g[4]) {
  if (tau <= 0.0 || sigma <= 0.0) {
    const double eq = exp(-q * tau);
    g[0] = put ? (S < K ? -eq : 0.0) : (S > K ? eq : 0.0);
    g[1] = g[2] = g[3] = 0.0;
    return;
  }
  const double sqt = sqrt(tau);
  const double d1 = (log(S / K) + (r - q + 0.5 * sigma * sigma) * tau) / (sigma * sqt);
  const double d2 = d1 - sigma * sqt;
  const double eq = exp(-q * tau), er = exp(-r * tau);
  const double pdf = norm_pdf(d1);
  g[1] = eq * pdf / (S * sigma * sqt);
  const double common = -S * eq * pdf * sigma / (2.0 * sqt);
  if (put) {
    g[0] = -eq * norm_cdf(-d1);
    g[2] = common + r * K * er * norm_cdf(-d2) - q * S * eq * norm_cdf(-d1);
    g[3] = -K * tau * er * norm_cdf(-d2);
  } else {
    g[0] = eq * norm_cdf(d1);
    g[2] = common - r * K * er * norm_cdf(d2) + q * S * eq * norm_cdf(d1);
    g[3] = K * tau * er * norm_cdf(d2);
  }
}

// eep_floor (eep_decomposer.hpp:21-29): debiased softplus with sharpness 100.
__device__ double eep_floor(double e) {
  if (100.0 * e > 500.0) return e;
  const double softplus = log1p(exp(100.0 * e)) / 100.0;
  const double bias = log(2.0) / 100.0;
  return fmax(0.0, softplus - bias);
}

}  // namespace

// One fit axis: slice s covers src[base + i * inner], i < n, with
// base = (s / inner) * n * inner + s % inner.  Factors in shared memory:
// band (4n), lower (3n), upper (7n) doubles, then col_start, piv (n each).
struct FitAxisDev {
  int n;
  int64_t inner;
  int64_t nslices;
};

__global__ void fit_axis_kernel(FitAxisDev A, const double* __restrict__ fac,
                                const int32_t* __restrict__ faci, const double* __restrict__ src,
                                double* __restrict__ dst, double tol,
                                unsigned long long* __restrict__ max_res_bits,
                                unsigned long long* __restrict__ failed) {
  extern __shared__ double fsm[];
  const int n = A.n;
  for (int i = threadIdx.x; i < 14 * n; i += blockDim.x) fsm[i] = fac[i];
  int32_t* ism = reinterpret_cast<int32_t*>(fsm + 14 * n);
  for (int i = threadIdx.x; i < 2 * n; i += blockDim.x) ism[i] = faci[i];
  __syncthreads();
  const double* band = fsm;
  const double* lower = fsm + 4 * n;
  const double* upper = fsm + 7 * n;
  const int32_t* col_start = ism;
  const int32_t* piv = ism + n;
  const int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  if (s >= A.nslices) return;
  const int64_t inner = A.inner;
  const int64_t base = (s / inner) * n * inner + s % inner;
  const double* f = src + base;
  double* c = dst + base;
  auto F = [&](int i) { return f[static_cast<size_t>(i) * inner]; };
  auto C = [&](int i) -> double& { return c[static_cast<size_t>(i) * inner]; };
  for (int i = 0; i < n; ++i) C(i) = F(i);
  // dgbtrs: forward elimination with the row interchanges
  for (int j = 0; j + 1 < n; ++j) {
    const int p = piv[j];
    if (p != j) {
      const double tmp = C(p);
      C(p) = C(j);
      C(j) = tmp;
    }
    const double bj = -C(j);
    const int lm = min(3, n - 1 - j);
    for (int i = 1; i <= lm; ++i) C(j + i) = __dadd_rn(C(j + i), __dmul_rn(lower[3 * j + i - 1], bj));
  }
  // dtbsv: column-oriented back substitution
  for (int j = n - 1; j >= 0; --j) {
    if (C(j) == 0.0) continue;
    const double cj = C(j) / upper[7 * j];
    C(j) = cj;
    for (int i = j - 1; i >= max(0, j - 6); --i)
      C(i) = __dsub_rn(C(i), __dmul_rn(cj, upper[7 * i + (j - i)]));
  }
  // compute_residual_from_span
  double res = 0.0;
  for (int i = 0; i < n; ++i) {
    double bc = 0.0;
    const int cs = col_start[i];
    for (int k = 0; k < 4 && cs + k < n; ++k) bc = fma(band[4 * i + k], C(cs + k), bc);
    res = fmax(res, fabs(bc - F(i)));
  }
  if (!(res <= tol)) {
    for (int i = 0; i < n; ++i) C(i) = F(i);
    atomicAdd(failed, 1ull);
  } else {
    atomicMax(max_res_bits, static_cast<unsigned long long>(__double_as_longlong(res)));
  }
}

// Tensor [m][tau][sigma][r] of V/K_ref -> EEP in price units.
__global__ void eep_decompose_kernel(int nm, int nt, int nv, int nr, const double* __restrict__ mg,
                                     const double* __restrict__ tg, const double* __restrict__ vg,
                                     const double* __restrict__ rg, double K_ref, double q, int put,
                                     double* __restrict__ tensor) {
  const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
  const int64_t total = static_cast<int64_t>(nm) * nt * nv * nr;
  if (i >= total) return;
  int64_t f = i;
  const int ri = static_cast<int>(f % nr);
  f /= nr;
  const int vi = static_cast<int>(f % nv);
  f /= nv;
  const int ti = static_cast<int>(f % nt);
  const int mi = static_cast<int>(f / nt);
  const double am = K_ref * tensor[i];
  const double spot = exp(mg[mi]) * K_ref;
  const double eu = european_price(spot, K_ref, tg[ti], vg[vi], rg[ri], q, put != 0);
  tensor[i] = eep_floor(am - eu);
}

// The table as the query kernels see it.
struct TableDev {
  double K_ref, q;
  int put, eep;
  double lo[4], hi[4];  // axis ranges (m, tau, sigma, rate)
};

// AnyPriceTable::price (EEPLayer::price over TransformLeaf::price).
__device__ __forceinline__ double table_price(const BSplineDims& D, const double* sm,
                                              const double* coeffs, const TableDev& T, double S,
                                              double K, double tau, double sigma, double r) {
  const double x[4] = {log(S / K), tau, sigma, r};
  const double raw = bspline4d_value(D, sm, coeffs, x);
  double v = fmax(0.0, raw) * K / T.K_ref;
  if (T.eep) v += european_price(S, K, tau, sigma, r, T.q, T.put != 0);
  return v;
}

// AnyPriceTable::vega (EEPLayer::vega over TransformLeaf::vega).
__device__ __forceinline__ double table_vega(const BSplineDims& D, const double* sm,
                                             const double* coeffs, const TableDev& T, double S,
                                             double K, double tau, double sigma, double r) {
  const double x[4] = {log(S / K), tau, sigma, r};
  const double raw = bspline4d_value(D, sm, coeffs, x);
  double v = 0.0;
  if (raw > 0.0) v = bspline4d_eval_t<2>(D, sm, coeffs, x) * K / T.K_ref;
  if (T.eep) v += european_vega(S, K, tau, sigma, r, T.q);
  return v;
}

__global__ void surface_vega_kernel(BSplineDims D, const double* __restrict__ tables,
                                    const double* __restrict__ coeffs, TableDev T,
                                    const MangoPricingParams* __restrict__ p, int64_t n,
                                    double* __restrict__ out) {
  extern __shared__ double sm[];
  for (int i = threadIdx.x; i < 4 * D.ktot; i += blockDim.x) sm[i] = tables[i];
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
    const MangoPricingParams pk = p[k];
    out[k] = pk.n_tenor_points != 0
                 ? __longlong_as_double(0x7ff8000000000000ll)
                 : table_vega(D, sm, coeffs, T, pk.spot, pk.strike, pk.maturity, pk.volatility,
                              pk.rate_const);
  }
}

// AnyPriceTable::delta/gamma/theta/rho behind the C API's greek_call
// (mango_c_api.cpp:272-300, 652-682): AnyPriceTable::validate_pricing_params
// (price_table_factory.cpp:700-745) first, then EEPLayer::greek / gamma
// (eep_layer.hpp:33-76) over TransformLeaf::greek / gamma
// (transform_leaf.hpp:46-90) with StandardTransform4D's weights
// (delta 1/S on axis 0, theta -1 on axis 1, rho 1 on axis 3) and
// gamma = (f_xx - f_x) / S^2, each scaled by K / K_ref.  A record that fails
// validation gets status MANGO_ERR_VALIDATION and NaN Greeks.
__global__ void surface_greeks_kernel(BSplineDims D, const double* __restrict__ tables,
                                      const double* __restrict__ coeffs, TableDev T,
                                      const MangoPricingParams* __restrict__ p, int64_t n,
                                      double* __restrict__ out4, int32_t* __restrict__ status) {
  extern __shared__ double sm[];
  for (int i = threadIdx.x; i < 4 * D.ktot; i += blockDim.x) sm[i] = tables[i];
  __syncthreads();
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
    const MangoPricingParams pk = p[k];
    const double S = pk.spot, K = pk.strike, tau = pk.maturity, sigma = pk.volatility,
                 r = pk.rate_const;
    const bool put = pk.option_type == MANGO_PUT;
    const double x[4] = {log(S / K), tau, sigma, r};
    const bool ok = (pk.option_type == MANGO_PUT || pk.option_type == MANGO_CALL) &&
                    pk.n_tenor_points == 0 && S > 0.0 && isfinite(S) && K > 0.0 && isfinite(K) &&
                    tau > 0.0 && isfinite(tau) && sigma > 0.0 && isfinite(sigma) && isfinite(r) &&
                    isfinite(pk.dividend_yield) && put == (T.put != 0) &&
                    fabs(pk.dividend_yield - T.q) <= 1e-10 && x[0] >= T.lo[0] && x[0] <= T.hi[0] &&
                    tau >= T.lo[1] && tau <= T.hi[1] && sigma >= T.lo[2] && sigma <= T.hi[2] &&
                    r >= T.lo[3] && r <= T.hi[3];
    double g[4] = {nan, nan, nan, nan};
    if (ok) {
      double e[4] = {0.0, 0.0, 0.0, 0.0};
      if (T.eep) european_greeks(S, K, tau, sigma, r, T.q, put, e);
      const double raw = bspline4d_value(D, sm, coeffs, x);
      if (raw > 0.0) {
        const double fx = bspline4d_eval_t<0>(D, sm, coeffs, x);
        const double fxx = bspline4d_eval_t<0, 2>(D, sm, coeffs, x);
        const double ft = bspline4d_eval_t<1>(D, sm, coeffs, x);
        const double fr = bspline4d_eval_t<3>(D, sm, coeffs, x);
        g[0] = __dmul_rn(1.0 / S, fx) * K / T.K_ref + e[0];
        g[1] = (fxx - fx) / (S * S) * K / T.K_ref + e[1];
        g[2] = -ft * K / T.K_ref + e[2];
        g[3] = fr * K / T.K_ref + e[3];
      } else {
        for (int j = 0; j < 4; ++j) g[j] = e[j];
      }
    }
    for (int j = 0; j < 4; ++j) out4[4 * k + j] = g[j];
    if (status) status[k] = ok ? MANGO_OK : MANGO_ERR_VALIDATION;
  }
}

// InterpolatedIVSolver::solve (interpolated_iv_solver.hpp:427-520) per quote.
__global__ void surface_iv_kernel(BSplineDims D, const double* __restrict__ tables,
                                  const double* __restrict__ coeffs, TableDev T,
                                  MangoInterpSolverConfig cfg,
                                  const MangoIvQuery* __restrict__ qs, int64_t n,
                                  MangoIvBatchSlot* __restrict__ out) {
  extern __shared__ double sm[];
  for (int i = threadIdx.x; i < 4 * D.ktot; i += blockDim.x) sm[i] = tables[i];
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
    const MangoIvQuery q = qs[k];
    MangoIvBatchSlot slot{};
    auto finish = [&](int32_t status) {
      slot.status = status;
      out[k] = slot;
    };
    // build_iv_query (mango_c_api.cpp:168-203) and validate_query
    // (interpolated_iv_solver.hpp:375-398): type and dividend yield must
    // match the table, then validate_iv_query.
    if (q.option_type != MANGO_PUT && q.option_type != MANGO_CALL) { finish(MANGO_ERR_VALIDATION); continue; }
    if (q.n_tenor_points != 0 || q.n_dividends != 0 || !isfinite(q.dividend_yield) ||
        !isfinite(q.rate_const)) { finish(MANGO_ERR_VALIDATION); continue; }
    const bool put = q.option_type == MANGO_PUT;
    if (put != (T.put != 0) || fabs(q.dividend_yield - T.q) > 1e-10) { finish(MANGO_ERR_VALIDATION); continue; }
    if (!(q.spot > 0.0) || !isfinite(q.spot) || !(q.strike > 0.0) || !isfinite(q.strike) ||
        !(q.maturity > 0.0) || !isfinite(q.maturity)) { finish(MANGO_ERR_VALIDATION); continue; }
    if (q.dividend_yield < 0.0) { finish(MANGO_ERR_ARBITRAGE); continue; }
    if (!isfinite(q.market_price) || q.market_price <= 0.0) { finish(MANGO_ERR_VALIDATION); continue; }
    const double intrinsic = put ? fmax(q.strike - q.spot, 0.0) : fmax(q.spot - q.strike, 0.0);
    const double upper_bound = put ? q.strike : q.spot;
    if (q.market_price < intrinsic || q.market_price > upper_bound) { finish(MANGO_ERR_ARBITRAGE); continue; }
    // adaptive_bounds (interpolated_iv_solver.hpp:400-425)
    const double tv_pct = (q.market_price - intrinsic) / q.market_price;
    const double sigma_upper = tv_pct > 0.5 ? 3.0 : (tv_pct > 0.2 ? 2.0 : 1.5);
    double smin = fmax(cfg.sigma_min, T.lo[2]);
    double smax = fmin(fmin(sigma_upper, cfg.sigma_max), T.hi[2]);
    if (smin >= smax) {
      smin = T.lo[2];
      smax = T.hi[2];
    }
    // is_in_bounds at both ends (interpolated_iv_solver.hpp:134-145)
    const double x = log(q.spot / q.strike);
    const double r = q.rate_const;
    const bool in = x >= T.lo[0] && x <= T.hi[0] && q.maturity >= T.lo[1] && q.maturity <= T.hi[1] &&
                    r >= T.lo[3] && r <= T.hi[3] && smin >= T.lo[2] && smin <= T.hi[2] &&
                    smax >= T.lo[2] && smax <= T.hi[2];
    if (!in) { finish(MANGO_ERR_VALIDATION); continue; }
    // vega pre-check
    if (cfg.vega_threshold > 0.0) {
      double vmax = 0.0;
      const double probe[3] = {0.10, 0.25, 0.50};
      for (int j = 0; j < 3; ++j)
        vmax = fmax(vmax, fabs(table_vega(D, sm, coeffs, T, q.spot, q.strike, q.maturity, probe[j], r)));
      if (vmax < cfg.vega_threshold) {
        slot.success.final_error = vmax;
        finish(MANGO_ERR_SOLVER);
        continue;
      }
    }
    // Brent on f(sigma) = price(m K, K, tau, sigma, r) - P
    const double mny = q.spot / q.strike;
    const double spot = mny * q.strike;
    BrentDev b;
    brentdev::brent_start(b, smin, smax);
    double sig = smin;
    const int max_iter = static_cast<int>(cfg.max_iter > 1000000 ? 1000000 : cfg.max_iter);
    for (int e = 0; e < max_iter + 3; ++e) {
      const double f = table_price(D, sm, coeffs, T, spot, q.strike, q.maturity, sig, r) - q.market_price;
      double next = 0.0;
      if (!brentdev::brent_consume(b, f, cfg.tolerance, max_iter, &next)) break;
      sig = next;
    }
    slot.success.iterations = static_cast<uint64_t>(b.iter);
    slot.success.final_error = b.ferr;
    if (b.code == kIvOk) {
      slot.success.implied_vol = b.root;
      finish(MANGO_OK);
    } else {
      finish(b.code == kIvBracket ? MANGO_ERR_BRACKETING
                                  : (b.code == kIvMaxIter ? MANGO_ERR_NO_CONVERGENCE : MANGO_ERR_SOLVER));
    }
  }
}

// AnyPriceTable::price for n parameter records.
__global__ void surface_price_kernel(BSplineDims D, const double* __restrict__ tables,
                                     const double* __restrict__ coeffs,
                                     const MangoPricingParams* __restrict__ p, int64_t n,
                                     double K_ref, double q, int put, int eep,
                                     double* __restrict__ out) {
  extern __shared__ double sm[];
  for (int i = threadIdx.x; i < 4 * D.ktot; i += blockDim.x) sm[i] = tables[i];
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; k < n; k += stride) {
    const MangoPricingParams pk = p[k];
    if (pk.n_tenor_points != 0) {  // get_zero_rate of a curve: not supported
      out[k] = __longlong_as_double(0x7ff8000000000000ll);
      continue;
    }
    const double S = pk.spot, K = pk.strike, tau = pk.maturity, sigma = pk.volatility;
    const double r = pk.rate_const;
    const double x[4] = {log(S / K), tau, sigma, r};
    const double raw = bspline4d_value(D, sm, coeffs, x);
    double v = fmax(0.0, raw) * K / K_ref;
    if (eep) v += european_price(S, K, tau, sigma, r, q, put != 0);
    out[k] = v;
  }
}

namespace {

// Fit the row-major tensor in a (n0*n1*n2*n3 doubles, device) in place; b is
// scratch of the same size.  Axis order 3, 2, 1, 0, ping-ponging a -> b -> a.
void fit_device(MangoGpuContext* ctx, const double* grids, const int64_t* sizes, double* a,
                double* b, double tol, MangoGpuFitStats* stats) {
  cudaStream_t st = ctx->stream;
  DevBuf d_fac, d_faci, d_acc;
  struct Release {
    DevBuf* d[3];
    ~Release() {
      for (DevBuf* x : d) x->release();
    }
  } release{{&d_fac, &d_faci, &d_acc}};
  unsigned long long* acc = static_cast<unsigned long long*>(d_acc.get(sizeof(unsigned long long) * 8));
  check(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 8, st), "memset");
  int64_t total = 1;
  for (int d = 0; d < 4; ++d) total *= sizes[d];
  int64_t offs[4];
  int64_t o = 0;
  for (int d = 0; d < 4; ++d) {
    offs[d] = o;
    o += sizes[d];
  }
  double* src = a;
  double* dst = b;
  std::vector<double> cond(4, 0.0);
  std::vector<int> singular(4, 0);
  for (int axis = 3; axis >= 0; --axis) {
    const int n = static_cast<int>(sizes[axis]);
    const AxisFactor F = factor_axis(grids + offs[axis], n);
    cond[axis] = F.cond1;
    int64_t inner = 1;
    for (int d = axis + 1; d < 4; ++d) inner *= sizes[d];
    const int64_t nslices = total / n;
    if (F.singular) {
      // factorize_banded_workspace fails for every slice: values stay.
      singular[axis] = 1;
      check(cudaMemcpyAsync(dst, src, sizeof(double) * total, cudaMemcpyDeviceToDevice, st), "D2D");
    } else {
      std::vector<double> fac(static_cast<size_t>(14) * n);
      std::vector<int32_t> faci(static_cast<size_t>(2) * n);
      std::copy(F.band.begin(), F.band.end(), fac.begin());
      std::copy(F.lower.begin(), F.lower.end(), fac.begin() + 4 * n);
      std::copy(F.upper.begin(), F.upper.end(), fac.begin() + 7 * n);
      std::copy(F.col_start.begin(), F.col_start.end(), faci.begin());
      std::copy(F.piv.begin(), F.piv.end(), faci.begin() + n);
      double* dfac = static_cast<double*>(d_fac.get(sizeof(double) * fac.size()));
      int32_t* dfaci = static_cast<int32_t*>(d_faci.get(sizeof(int32_t) * faci.size()));
      check(cudaMemcpyAsync(dfac, fac.data(), sizeof(double) * fac.size(), cudaMemcpyHostToDevice, st), "H2D");
      check(cudaMemcpyAsync(dfaci, faci.data(), sizeof(int32_t) * faci.size(), cudaMemcpyHostToDevice, st), "H2D");
      const size_t smem = sizeof(double) * 14 * n + sizeof(int32_t) * 2 * n;
      check(cudaFuncSetAttribute(fit_axis_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)),
            "smem attribute");
      const int tb = 128;
      fit_axis_kernel<<<static_cast<int>((nslices + tb - 1) / tb), tb, smem, st>>>(
          FitAxisDev{n, inner, nslices}, dfac, dfaci, src, dst, tol, acc + axis, acc + 4 + axis);
      check(cudaGetLastError(), "fit_axis_kernel launch");
      // the host vectors must outlive the copies
      check(cudaStreamSynchronize(st), "stream synchronize");
    }
    std::swap(src, dst);
  }
  unsigned long long h[8];
  check(cudaMemcpyAsync(h, acc, sizeof(h), cudaMemcpyDeviceToHost, st), "D2H");
  check(cudaStreamSynchronize(st), "stream synchronize");
  if (stats) {
    for (int d = 0; d < 4; ++d) {
      double r;
      std::memcpy(&r, &h[d], sizeof(r));
      stats->max_residual[d] = r;
      stats->condition[d] = cond[d];
      stats->failed_slices[d] = singular[d] ? static_cast<uint64_t>(total / sizes[d]) : h[4 + d];
    }
  }
}

uint64_t total_failed(const MangoGpuFitStats& s) {
  return s.failed_slices[0] + s.failed_slices[1] + s.failed_slices[2] + s.failed_slices[3];
}

std::string check_fit_args(const double* grids, const int64_t* sizes, int64_t* total) {
  if (!grids || !sizes) return "null grids or sizes";
  *total = 1;
  for (int d = 0; d < 4; ++d) {
    if (sizes[d] < 4 || sizes[d] > kMaxAxis) return "each axis needs 4..512 grid points";
    *total *= sizes[d];
  }
  return {};
}

}  // namespace
}  // namespace mgpu

struct MangoGpuPriceTable {
  MangoGpuBSpline4D* surface = nullptr;
  double K_ref = 0, q = 0;
  int32_t option_type = 0;
  int32_t eep = 1;
  double bounds[8] = {};  // m, tau, sigma, rate: min, max
  mgpu::DevBuf d_p, d_out;
};

using namespace mgpu;

extern "C" {

MangoStatus mango_gpu_bspline4d_fit(MangoGpuContext* ctx, const double* grids,
                                    const int64_t* sizes, const double* values, double tolerance,
                                    double* coeffs, MangoGpuFitStats* stats, MangoError* err) {
  int64_t total = 0;
  std::string bad = check_fit_args(grids, sizes, &total);
  if (!ctx || !values || !coeffs) bad = "null argument";
  if (!bad.empty()) {
    set_err(err, MANGO_ERR_VALIDATION, bad);
    return MANGO_ERR_VALIDATION;
  }
  for (int64_t i = 0; i < total; ++i)
    if (!std::isfinite(values[i])) {
      set_err(err, MANGO_ERR_VALIDATION, std::isnan(values[i]) ? "NaN input value" : "infinite input value");
      return MANGO_ERR_VALIDATION;
    }
  DevBuf da, db;
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    {  // BSplineNDSeparable::create validation: strictly increasing axes
      std::vector<double> tab, kn;
      BSplineDims D;
      bspline_tables(grids, sizes, &D, &tab, &kn);
    }
    cudaStream_t st = ctx->stream;
    double* a = static_cast<double*>(da.get(sizeof(double) * total));
    double* b = static_cast<double*>(db.get(sizeof(double) * total));
    check(cudaMemcpyAsync(a, values, sizeof(double) * total, cudaMemcpyHostToDevice, st), "H2D");
    MangoGpuFitStats s{};
    fit_device(ctx, grids, sizes, a, b, tolerance > 0.0 ? tolerance : 1e-6, &s);
    check(cudaMemcpyAsync(coeffs, a, sizeof(double) * total, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    da.release();
    db.release();
    if (stats) *stats = s;
    if (total_failed(s) > 0) {
      set_err(err, MANGO_ERR_SOLVER, "fitting failed: " + std::to_string(total_failed(s)) + " slices");
      return MANGO_ERR_SOLVER;
    }
    return MANGO_OK;
  } catch (const std::invalid_argument& e) {
    da.release();
    db.release();
    set_err(err, MANGO_ERR_VALIDATION, e.what());
    return MANGO_ERR_VALIDATION;
  } catch (const std::exception& e) {
    da.release();
    db.release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_price_table_create(MangoGpuContext* ctx, const double* grids,
                                         const int64_t* sizes, const double* coeffs, double K_ref,
                                         double dividend_yield, MangoOptionType option_type,
                                         int32_t eep, MangoGpuPriceTable** out, MangoError* err) {
  if (out) *out = nullptr;
  MangoGpuBSpline4D* s = nullptr;
  MangoStatus rc = mango_gpu_bspline4d_create(ctx, grids, sizes, coeffs, &s, err);
  if (rc != MANGO_OK) return rc;
  if (!out || !(K_ref > 0.0) || (option_type != MANGO_PUT && option_type != MANGO_CALL)) {
    mango_gpu_bspline4d_destroy(s);
    set_err(err, MANGO_ERR_VALIDATION, "invalid K_ref, option type or out");
    return MANGO_ERR_VALIDATION;
  }
  MangoGpuPriceTable* t = new MangoGpuPriceTable();
  t->surface = s;
  t->K_ref = K_ref;
  t->q = dividend_yield;
  t->option_type = option_type;
  t->eep = eep ? 1 : 0;
  for (int d = 0; d < 4; ++d) {
    t->bounds[2 * d] = s->dims.lo[d];
    t->bounds[2 * d + 1] = s->dims.hi[d];
  }
  *out = t;
  return MANGO_OK;
}

}  // extern "C"

namespace mgpu {
namespace {

// PriceTableBuilderND<4>'s failure handling on the swept tensor
// [m][tau][sigma][r] (host copy), as the reference runs it after the sweep
// (src/option/table/bspline/bspline_builder.cpp:95-101, 773-959).  A slice
// (sigma, r) whose every entry is NaN failed as a whole (its PDE solve, or
// the spline resampling at every maturity); a slice with NaN at some
// maturities failed there only.  Those maturities are interpolated linearly
// along tau from the nearest valid maturities of the same slice (or copied
// from the one valid side); whole slices are copied from the nearest valid
// (sigma, r) slice in Manhattan distance, searched dist = 1, 2, ... with
// dsigma from -dist to dist and the rate offset's sign -, + (a repaired slice
// then counts as a donor).  The reference visits whole-slice failures in a
// hash set's order; here they go in ascending (sigma, r) order.
// Returns the whole slices and the (slice, maturity) points repaired; throws
// when a slice has no valid neighbour.
std::pair<uint64_t, uint64_t> repair_tensor(std::vector<double>& ten, int64_t nm, int64_t nt,
                                            int64_t ns, int64_t nr) {
  auto at = [&](int64_t i, int64_t j, int64_t s, int64_t r) -> double& {
    return ten[((i * nt + j) * ns + s) * nr + r];
  };
  const int64_t nslice = ns * nr;
  std::vector<char> full(static_cast<size_t>(nslice), 0);
  std::vector<std::vector<int64_t>> partial(static_cast<size_t>(nslice));
  for (int64_t s = 0; s < ns; ++s)
    for (int64_t r = 0; r < nr; ++r) {
      int64_t bad = 0;
      for (int64_t j = 0; j < nt; ++j) {
        bool nanj = false;
        for (int64_t i = 0; i < nm && !nanj; ++i) nanj = std::isnan(at(i, j, s, r));
        if (nanj) {
          partial[s * nr + r].push_back(j);
          ++bad;
        }
      }
      if (bad == nt) full[s * nr + r] = 1;
    }
  uint64_t points = 0;
  for (int64_t k = 0; k < nslice; ++k) {
    if (full[k] || partial[k].empty()) continue;
    const int64_t s = k / nr, r = k % nr;
    for (int64_t j : partial[k]) {
      int64_t before = -1, after = -1;
      for (int64_t q = j; q-- > 0;)
        if (!std::isnan(at(0, q, s, r))) {
          before = q;
          break;
        }
      for (int64_t q = j + 1; q < nt; ++q)
        if (!std::isnan(at(0, q, s, r))) {
          after = q;
          break;
        }
      for (int64_t i = 0; i < nm; ++i) {
        if (before >= 0 && after >= 0) {
          const double w = static_cast<double>(j - before) / static_cast<double>(after - before);
          at(i, j, s, r) = (1.0 - w) * at(i, before, s, r) + w * at(i, after, s, r);
        } else {
          at(i, j, s, r) = at(i, before >= 0 ? before : after, s, r);
        }
      }
      ++points;
    }
  }
  std::vector<char> valid(static_cast<size_t>(nslice));
  for (int64_t k = 0; k < nslice; ++k) valid[k] = !full[k];
  uint64_t slices = 0;
  for (int64_t k = 0; k < nslice; ++k) {
    if (!full[k]) continue;
    const int64_t s = k / nr, r = k % nr;
    int64_t ds_found = -1, dr_found = -1;
    for (int64_t dist = 1; dist <= (ns - 1) + (nr - 1) && ds_found < 0; ++dist)
      for (int64_t dsg = -dist; dsg <= dist && ds_found < 0; ++dsg) {
        const int64_t drr = dist - (dsg < 0 ? -dsg : dsg);
        for (int sign : {-1, 1}) {
          const int64_t s2 = s + dsg, r2 = r + sign * drr;
          if (s2 >= 0 && s2 < ns && r2 >= 0 && r2 < nr && valid[s2 * nr + r2]) {
            ds_found = s2;
            dr_found = r2;
            break;
          }
        }
      }
    if (ds_found < 0)
      throw std::runtime_error("failed-slice repair: slice " + std::to_string(k) +
                               " has no valid neighbour");
    for (int64_t i = 0; i < nm; ++i)
      for (int64_t j = 0; j < nt; ++j) at(i, j, s, r) = at(i, j, ds_found, dr_found);
    valid[k] = 1;
    ++slices;
  }
  return {slices, points};
}

// Test hook, host side: MANGO_GPU_TABLE_FAIL="k,k:j,..." reports slice k
// (flat sigma * n_rate + r) as failed as a whole, or at maturity j only, as
// if its solve or its resampling had failed; the repair then runs on it.
// Nothing on the device is altered.
uint64_t inject_table_failures(std::vector<double>& ten, int64_t nm, int64_t nt, int64_t ns,
                               int64_t nr) {
  const char* e = std::getenv("MANGO_GPU_TABLE_FAIL");
  if (!e || !*e) return 0;
  uint64_t whole = 0;
  std::string spec(e);
  size_t pos = 0;
  while (pos < spec.size()) {
    size_t end = spec.find(',', pos);
    if (end == std::string::npos) end = spec.size();
    const std::string item = spec.substr(pos, end - pos);
    pos = end + 1;
    if (item.empty()) continue;
    const size_t colon = item.find(':');
    const int64_t k = std::stoll(item.substr(0, colon));
    if (k < 0 || k >= ns * nr) continue;
    const int64_t s = k / nr, r = k % nr;
    const double nan = std::nan("");
    if (colon == std::string::npos) {
      for (int64_t i = 0; i < nm; ++i)
        for (int64_t j = 0; j < nt; ++j) ten[((i * nt + j) * ns + s) * nr + r] = nan;
      ++whole;
    } else {
      const int64_t j = std::stoll(item.substr(colon + 1));
      if (j < 0 || j >= nt) continue;
      for (int64_t i = 0; i < nm; ++i) ten[((i * nt + j) * ns + s) * nr + r] = nan;
    }
  }
  return whole;
}

}  // namespace
}  // namespace mgpu

extern "C" {

MangoStatus mango_gpu_price_table_build(
    MangoGpuContext* ctx, const double* moneyness, uint64_t nm, const double* maturity,
    uint64_t ntau, const double* volatility, uint64_t nsig, const double* rate, uint64_t nr,
    double K_ref, double dividend_yield, MangoOptionType option_type, const MangoGpuGrid* grid,
    int32_t eep, double tolerance, MangoGpuPriceTable** out, MangoGpuFitStats* stats,
    uint64_t* out_failed_slices, MangoError* err) {
  return mango_gpu_price_table_build_ex(ctx, moneyness, nm, maturity, ntau, volatility, nsig, rate,
                                        nr, K_ref, dividend_yield, option_type, grid, eep,
                                        tolerance, 0.0, out, stats, out_failed_slices, nullptr,
                                        err);
}

MangoStatus mango_gpu_price_table_build_ex(
    MangoGpuContext* ctx, const double* moneyness, uint64_t nm, const double* maturity,
    uint64_t ntau, const double* volatility, uint64_t nsig, const double* rate, uint64_t nr,
    double K_ref, double dividend_yield, MangoOptionType option_type, const MangoGpuGrid* grid,
    int32_t eep, double tolerance, double max_failure_rate, MangoGpuPriceTable** out,
    MangoGpuFitStats* stats, uint64_t* out_failed_slices, uint64_t* out_repaired,
    MangoError* err) {
  if (out) *out = nullptr;
  if (out_repaired) out_repaired[0] = out_repaired[1] = 0;
  if (!(max_failure_rate >= 0.0 && max_failure_rate <= 1.0)) {
    // PriceTableConfig validation (bspline_builder.hpp:108-111)
    set_err(err, MANGO_ERR_VALIDATION, "max_failure_rate must be in [0.0, 1.0]");
    return MANGO_ERR_VALIDATION;
  }
  std::string bad = check_table_args(moneyness, nm, maturity, ntau, volatility, nsig, rate, nr,
                                     K_ref, dividend_yield, option_type);
  if (bad.empty() && (!ctx || !out)) bad = "null argument";
  const int64_t sizes[4] = {static_cast<int64_t>(nm), static_cast<int64_t>(ntau),
                            static_cast<int64_t>(nsig), static_cast<int64_t>(nr)};
  std::vector<double> grids;
  if (bad.empty()) {
    grids.insert(grids.end(), moneyness, moneyness + nm);
    grids.insert(grids.end(), maturity, maturity + ntau);
    grids.insert(grids.end(), volatility, volatility + nsig);
    grids.insert(grids.end(), rate, rate + nr);
    int64_t total = 0;
    bad = check_fit_args(grids.data(), sizes, &total);
  }
  if (!bad.empty()) {
    set_err(err, MANGO_ERR_VALIDATION, bad);
    return MANGO_ERR_VALIDATION;
  }
  MangoGpuPriceTable* t = nullptr;
  DevBuf da, db, dax;
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    t = new MangoGpuPriceTable();
    t->surface = new_surface(ctx, grids.data(), sizes);
    t->K_ref = K_ref;
    t->q = dividend_yield;
    t->option_type = option_type;
    t->eep = eep ? 1 : 0;
    for (int d = 0; d < 4; ++d) {
      t->bounds[2 * d] = t->surface->dims.lo[d];
      t->bounds[2 * d + 1] = t->surface->dims.hi[d];
    }
    cudaStream_t st = ctx->stream;
    const int64_t total = static_cast<int64_t>(nm * ntau * nsig * nr);
    double* a = static_cast<double*>(da.get(sizeof(double) * total));
    double* b = static_cast<double*>(db.get(sizeof(double) * total));
    // Step 1: sweep + extraction into a.
    const uint64_t failed = table_sweep_device(ctx, moneyness, nm, maturity, ntau, volatility, nsig,
                                               rate, nr, K_ref, dividend_yield, option_type, grid,
                                               a, nullptr);
    // Failure rate and repair (bspline_builder.cpp:95-101, 773-959) on a
    // host copy of the tensor (nm x ntau x nsig x nr doubles, a few MB); it
    // goes back to the device only when some entry was NaN (a failed solve
    // or resampling, or the host-side test hook) and has been repaired.
    {
      std::vector<double> ten(static_cast<size_t>(total));
      check(cudaMemcpyAsync(ten.data(), a, sizeof(double) * total, cudaMemcpyDeviceToHost, st),
            "D2H tensor");
      check(cudaStreamSynchronize(st), "stream synchronize");
      const uint64_t injected = inject_table_failures(ten, static_cast<int64_t>(nm),
                                                      static_cast<int64_t>(ntau),
                                                      static_cast<int64_t>(nsig),
                                                      static_cast<int64_t>(nr));
      const uint64_t pde_failed = failed + injected;
      if (out_failed_slices) *out_failed_slices = pde_failed;
      const double rate_failed =
          static_cast<double>(pde_failed) / static_cast<double>(nsig * nr);
      if (rate_failed > max_failure_rate)
        throw std::runtime_error(std::to_string(pde_failed) + " of " +
                                 std::to_string(nsig * nr) +
                                 " PDE slices failed, above max_failure_rate");
      bool any_nan = false;
      for (double v : ten)
        if (std::isnan(v)) {
          any_nan = true;
          break;
        }
      if (any_nan) {
        const auto rep = repair_tensor(ten, static_cast<int64_t>(nm), static_cast<int64_t>(ntau),
                                       static_cast<int64_t>(nsig), static_cast<int64_t>(nr));
        if (out_repaired) {
          out_repaired[0] = rep.first;
          out_repaired[1] = rep.second;
        }
        check(cudaMemcpyAsync(a, ten.data(), sizeof(double) * total, cudaMemcpyHostToDevice, st),
              "H2D repaired tensor");
        check(cudaStreamSynchronize(st), "stream synchronize");
      }
    }
    // Step 3: EEP decomposition.
    if (t->eep) {
      double* ax = static_cast<double*>(dax.get(sizeof(double) * grids.size()));
      check(cudaMemcpyAsync(ax, grids.data(), sizeof(double) * grids.size(), cudaMemcpyHostToDevice, st), "H2D");
      const int tb = 256;
      eep_decompose_kernel<<<static_cast<int>((total + tb - 1) / tb), tb, 0, st>>>(
          static_cast<int>(nm), static_cast<int>(ntau), static_cast<int>(nsig), static_cast<int>(nr),
          ax, ax + nm, ax + nm + ntau, ax + nm + ntau + nsig, K_ref, dividend_yield,
          option_type == MANGO_PUT ? 1 : 0, a);
      check(cudaGetLastError(), "eep_decompose_kernel launch");
    }
    // Step 4: fit (results in a); step 5: the surface takes them over.
    MangoGpuFitStats s{};
    fit_device(ctx, grids.data(), sizes, a, b, tolerance > 0.0 ? tolerance : 1e-6, &s);
    if (stats) *stats = s;
    if (total_failed(s) > 0)
      throw std::runtime_error("fitting failed: " + std::to_string(total_failed(s)) + " slices");
    std::swap(t->surface->d_coeffs.p, da.p);
    std::swap(t->surface->d_coeffs.cap, da.cap);
    db.release();
    da.release();
    dax.release();
    *out = t;
    return MANGO_OK;
  } catch (const std::exception& e) {
    da.release();
    db.release();
    dax.release();
    if (t) {
      if (t->surface) mango_gpu_bspline4d_destroy(t->surface);
      delete t;
    }
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_eep_decompose(MangoGpuContext* ctx, const double* moneyness, uint64_t nm,
                                    const double* maturity, uint64_t ntau,
                                    const double* volatility, uint64_t nsig, const double* rate,
                                    uint64_t nr, double K_ref, double dividend_yield,
                                    MangoOptionType option_type, double* tensor, MangoError* err) {
  std::string bad = check_table_args(moneyness, nm, maturity, ntau, volatility, nsig, rate, nr,
                                     K_ref, dividend_yield, option_type);
  if (bad.empty() && (!ctx || !tensor)) bad = "null argument";
  if (!bad.empty()) {
    set_err(err, MANGO_ERR_VALIDATION, bad);
    return MANGO_ERR_VALIDATION;
  }
  DevBuf dt, dax;
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t st = ctx->stream;
    const int64_t total = static_cast<int64_t>(nm * ntau * nsig * nr);
    std::vector<double> ax;
    ax.insert(ax.end(), moneyness, moneyness + nm);
    ax.insert(ax.end(), maturity, maturity + ntau);
    ax.insert(ax.end(), volatility, volatility + nsig);
    ax.insert(ax.end(), rate, rate + nr);
    double* d = static_cast<double*>(dt.get(sizeof(double) * total));
    double* a = static_cast<double*>(dax.get(sizeof(double) * ax.size()));
    check(cudaMemcpyAsync(d, tensor, sizeof(double) * total, cudaMemcpyHostToDevice, st), "H2D");
    check(cudaMemcpyAsync(a, ax.data(), sizeof(double) * ax.size(), cudaMemcpyHostToDevice, st), "H2D");
    const int tb = 256;
    eep_decompose_kernel<<<static_cast<int>((total + tb - 1) / tb), tb, 0, st>>>(
        static_cast<int>(nm), static_cast<int>(ntau), static_cast<int>(nsig), static_cast<int>(nr), a,
        a + nm, a + nm + ntau, a + nm + ntau + nsig, K_ref, dividend_yield,
        option_type == MANGO_PUT ? 1 : 0, d);
    check(cudaGetLastError(), "eep_decompose_kernel launch");
    check(cudaMemcpyAsync(tensor, d, sizeof(double) * total, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    dt.release();
    dax.release();
    return MANGO_OK;
  } catch (const std::exception& e) {
    dt.release();
    dax.release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

void mango_gpu_price_table_destroy(MangoGpuPriceTable* t) {
  if (!t) return;
  if (t->surface) {
    cudaSetDevice(t->surface->ctx->device);
    cudaStreamSynchronize(t->surface->ctx->stream);
  }
  t->d_p.release();
  t->d_out.release();
  if (t->surface) mango_gpu_bspline4d_destroy(t->surface);
  delete t;
}

MangoGpuBSpline4D* mango_gpu_price_table_spline(MangoGpuPriceTable* t) {
  return t ? t->surface : nullptr;
}

MangoStatus mango_gpu_price_table_info(const MangoGpuPriceTable* t, double* K_ref,
                                       double* dividend_yield, int32_t* option_type,
                                       int32_t* eep, double* bounds8) {
  if (!t) return MANGO_ERR_VALIDATION;
  if (K_ref) *K_ref = t->K_ref;
  if (dividend_yield) *dividend_yield = t->q;
  if (option_type) *option_type = t->option_type;
  if (eep) *eep = t->eep;
  if (bounds8) std::memcpy(bounds8, t->bounds, sizeof(t->bounds));
  return MANGO_OK;
}

MangoStatus mango_gpu_price_table_price_device(MangoGpuPriceTable* t,
                                               const MangoPricingParams* d_params, uint64_t n,
                                               double* d_out, MangoError* err) {
  if (!t || (n > 0 && (!d_params || !d_out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    MangoGpuBSpline4D* s = t->surface;
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    const int64_t need = static_cast<int64_t>((n + 255) / 256);
    const int blocks = static_cast<int>(std::min<int64_t>(s->blocks, need));
    surface_price_kernel<<<blocks, 256, sizeof(double) * 4 * s->dims.ktot, s->ctx->stream>>>(
        s->dims, s->d_tables.as<double>(), s->d_coeffs.as<double>(), d_params,
        static_cast<int64_t>(n), t->K_ref, t->q, t->option_type == MANGO_PUT ? 1 : 0, t->eep, d_out);
    check(cudaGetLastError(), "surface_price_kernel launch");
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_price_table_price(MangoGpuPriceTable* t, const MangoPricingParams* params,
                                        uint64_t n, double* out, MangoError* err) {
  if (!t || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    MangoGpuBSpline4D* s = t->surface;
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    MangoPricingParams* dp = static_cast<MangoPricingParams*>(t->d_p.get(sizeof(MangoPricingParams) * n));
    double* dout = static_cast<double*>(t->d_out.get(sizeof(double) * n));
    check(cudaMemcpyAsync(dp, params, sizeof(MangoPricingParams) * n, cudaMemcpyHostToDevice, st), "H2D");
    MangoStatus rc = mango_gpu_price_table_price_device(t, dp, n, dout, err);
    if (rc != MANGO_OK) return rc;
    check(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

}  // extern "C"

namespace {

TableDev table_dev(const MangoGpuPriceTable* t) {
  TableDev T{};
  T.K_ref = t->K_ref;
  T.q = t->q;
  T.put = t->option_type == MANGO_PUT ? 1 : 0;
  T.eep = t->eep;
  for (int d = 0; d < 4; ++d) {
    T.lo[d] = t->bounds[2 * d];
    T.hi[d] = t->bounds[2 * d + 1];
  }
  return T;
}

MangoInterpSolverConfig interp_config(const MangoInterpSolverConfig* c) {
  if (c) return *c;
  MangoInterpSolverConfig d{};
  d.max_iter = 50;  // InterpolatedIVSolverConfig (interpolated_iv_solver.hpp:44-57)
  d.tolerance = 1e-6;
  d.sigma_min = 0.01;
  d.sigma_max = 3.0;
  d.vega_threshold = 1e-4;
  return d;
}

}  // namespace

extern "C" {

MangoStatus mango_gpu_price_table_vega(MangoGpuPriceTable* t, const MangoPricingParams* params,
                                       uint64_t n, double* out, MangoError* err) {
  if (!t || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    MangoGpuBSpline4D* s = t->surface;
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    MangoPricingParams* dp = static_cast<MangoPricingParams*>(t->d_p.get(sizeof(MangoPricingParams) * n));
    double* dout = static_cast<double*>(t->d_out.get(sizeof(double) * n));
    check(cudaMemcpyAsync(dp, params, sizeof(MangoPricingParams) * n, cudaMemcpyHostToDevice, st), "H2D");
    const int blocks = static_cast<int>(std::min<int64_t>(s->blocks, static_cast<int64_t>((n + 255) / 256)));
    surface_vega_kernel<<<blocks, 256, sizeof(double) * 4 * s->dims.ktot, st>>>(
        s->dims, s->d_tables.as<double>(), s->d_coeffs.as<double>(), table_dev(t), dp,
        static_cast<int64_t>(n), dout);
    check(cudaGetLastError(), "surface_vega_kernel launch");
    check(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_price_table_greeks(MangoGpuPriceTable* t, const MangoPricingParams* params,
                                         uint64_t n, double* out4, int32_t* status,
                                         MangoError* err) {
  if (!t || (n > 0 && (!params || !out4))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    MangoGpuBSpline4D* s = t->surface;
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    const size_t pb = sizeof(MangoPricingParams) * n;
    MangoPricingParams* dp = static_cast<MangoPricingParams*>(t->d_p.get(pb));
    // Greeks (4n doubles) then the statuses (n int32) in one buffer.
    char* dbuf = static_cast<char*>(t->d_out.get(sizeof(double) * 4 * n + sizeof(int32_t) * n));
    double* dout = reinterpret_cast<double*>(dbuf);
    int32_t* dst = reinterpret_cast<int32_t*>(dbuf + sizeof(double) * 4 * n);
    check(cudaMemcpyAsync(dp, params, pb, cudaMemcpyHostToDevice, st), "H2D");
    const int blocks = static_cast<int>(std::min<int64_t>(s->blocks, static_cast<int64_t>((n + 255) / 256)));
    surface_greeks_kernel<<<blocks, 256, sizeof(double) * 4 * s->dims.ktot, st>>>(
        s->dims, s->d_tables.as<double>(), s->d_coeffs.as<double>(), table_dev(t), dp,
        static_cast<int64_t>(n), dout, dst);
    check(cudaGetLastError(), "surface_greeks_kernel launch");
    check(cudaMemcpyAsync(out4, dout, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, st), "D2H");
    std::vector<int32_t> hs(n);
    check(cudaMemcpyAsync(hs.data(), dst, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    uint64_t bad = 0, first = 0;
    for (uint64_t i = 0; i < n; ++i)
      if (hs[i] != MANGO_OK && bad++ == 0) first = i;
    if (status) std::memcpy(status, hs.data(), sizeof(int32_t) * n);
    if (bad) {
      const std::string msg = std::to_string(bad) + " record(s) failed validation (type, dividend "
                              "yield, positivity or table range), first at index " +
                              std::to_string(first);
      set_err(err, MANGO_ERR_VALIDATION, msg.c_str());
      return MANGO_ERR_VALIDATION;
    }
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_price_table_iv_batch_device(MangoGpuPriceTable* t,
                                                  const MangoInterpSolverConfig* config,
                                                  const MangoIvQuery* d_queries, uint64_t n,
                                                  MangoIvBatchSlot* d_out, MangoError* err) {
  if (!t || (n > 0 && (!d_queries || !d_out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    MangoGpuBSpline4D* s = t->surface;
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    const int blocks = static_cast<int>(std::min<int64_t>(s->blocks, static_cast<int64_t>((n + 255) / 256)));
    surface_iv_kernel<<<blocks, 256, sizeof(double) * 4 * s->dims.ktot, s->ctx->stream>>>(
        s->dims, s->d_tables.as<double>(), s->d_coeffs.as<double>(), table_dev(t), interp_config(config),
        d_queries, static_cast<int64_t>(n), d_out);
    check(cudaGetLastError(), "surface_iv_kernel launch");
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_price_table_iv_batch(MangoGpuPriceTable* t,
                                           const MangoInterpSolverConfig* config,
                                           const MangoIvQuery* queries, uint64_t n,
                                           MangoIvBatchSlot* out, uint64_t* out_failed,
                                           MangoError* err) {
  if (!t || (n > 0 && (!queries || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (out_failed) *out_failed = 0;
  if (n == 0) return MANGO_OK;
  DevBuf dq, ds;
  try {
    MangoGpuBSpline4D* s = t->surface;
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    MangoIvQuery* d_q = static_cast<MangoIvQuery*>(dq.get(sizeof(MangoIvQuery) * n));
    MangoIvBatchSlot* d_s = static_cast<MangoIvBatchSlot*>(ds.get(sizeof(MangoIvBatchSlot) * n));
    check(cudaMemcpyAsync(d_q, queries, sizeof(MangoIvQuery) * n, cudaMemcpyHostToDevice, st), "H2D");
    MangoStatus rc = mango_gpu_price_table_iv_batch_device(t, config, d_q, n, d_s, err);
    if (rc != MANGO_OK) {
      dq.release();
      ds.release();
      return rc;
    }
    check(cudaMemcpyAsync(out, d_s, sizeof(MangoIvBatchSlot) * n, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "stream synchronize");
    dq.release();
    ds.release();
    uint64_t failed = 0;
    for (uint64_t i = 0; i < n; ++i) failed += out[i].status != MANGO_OK;
    if (out_failed) *out_failed = failed;
    return MANGO_OK;
  } catch (const std::exception& e) {
    dq.release();
    ds.release();
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

}  // extern "C"
