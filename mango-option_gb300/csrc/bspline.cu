// bspline.cu -- 4D cubic B-spline surface query on the GPU.
//
// BSplineND<double,4> (src/math/bspline/bspline_nd.hpp) behind the C ABI:
// knots from clamped_knots_cubic (src/math/bspline/bspline_basis.hpp:47-91),
// evaluation in bspline.cuh.  GB300 design: one thread per query, FP64
// throughout; knots and the reciprocals of every Cox-de Boor denominator
// live in shared memory, so the basis needs no divide; the coefficient table
// (2.4 MB at 50x30x20x10) stays in L2 and is read through the read-only path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "bspline.cuh"

namespace mgpu {

std::vector<double> clamped_knots(const double* x, int n) {
  std::vector<double> t(static_cast<size_t>(n) + 4);
  std::fill_n(t.begin(), 4, x[0]);
  if (n > 4) {
    const int interior = n - 4, intervals = n - 1;
    for (int idx = 0; idx < interior; ++idx) {
      const double ratio = static_cast<double>(idx + 1) / static_cast<double>(interior + 1);
      const double pos = ratio * static_cast<double>(intervals);
      int low = static_cast<int>(std::floor(pos));
      if (low >= intervals) low = intervals - 1;
      const double frac = pos - static_cast<double>(low);
      const double left = x[low], right = x[low + 1];
      double knot = (1.0 - frac) * left + frac * right;
      const double spacing = right - left;
      const double eps = std::max(128.0 * DBL_EPSILON * spacing,
                                  DBL_EPSILON * std::max(std::fabs(right), 1.0));
      knot = std::clamp(knot, left + eps, right - eps);
      t[4 + idx] = knot;
    }
  }
  std::fill_n(t.end() - 4, 4, x[n - 1]);
  return t;
}

void bspline_tables(const double* grids, const int64_t* sizes, BSplineDims* Dp,
                    std::vector<double>* tab, std::vector<double>* knots) {
  BSplineDims& D = *Dp;
  int koff = 0;
  const double* g = grids;
  std::vector<std::vector<double>> kn(4);
  for (int d = 0; d < 4; ++d) {
    if (sizes[d] < 4 || sizes[d] > kMaxAxis)
      throw std::invalid_argument("each axis needs 4..512 grid points");
    const int n = static_cast<int>(sizes[d]);
    for (int i = 0; i < n; ++i)
      if (!std::isfinite(g[i])) throw std::invalid_argument("non-finite grid point");
    for (int i = 1; i < n; ++i)
      if (!(g[i] > g[i - 1])) throw std::invalid_argument("grid axes must be strictly increasing");
    kn[d] = clamped_knots(g, n);
    D.n[d] = n;
    D.koff[d] = koff;
    koff += n + 4;
    D.lo[d] = g[0];
    D.hi[d] = g[n - 1];
    D.hi_below[d] = std::nextafter(g[n - 1], -INFINITY);
    D.tlast[d] = kn[d].back();
    g += n;
  }
  D.ktot = koff;
  tab->assign(static_cast<size_t>(4 * koff), 0.0);
  knots->clear();
  for (int d = 0; d < 4; ++d) {
    const std::vector<double>& t = kn[d];
    const int nk = static_cast<int>(t.size());
    for (int j = 0; j < nk; ++j) {
      (*tab)[D.koff[d] + j] = t[j];
      knots->push_back(t[j]);
      for (int deg = 1; deg <= 3; ++deg) {
        double r = 0.0;
        if (j + deg < nk) {
          const double den = t[j + deg] - t[j];
          if (den > 0.0) r = 1.0 / den;
        }
        (*tab)[static_cast<size_t>(deg) * koff + D.koff[d] + j] = r;
      }
    }
  }
}

__global__ void bspline4d_eval_kernel(BSplineDims D, const double* __restrict__ tables,
                                      const double* __restrict__ coeffs,
                                      const double* __restrict__ q, int64_t nq,
                                      double* __restrict__ out) {
  extern __shared__ double sm[];
  for (int i = threadIdx.x; i < 4 * D.ktot; i += blockDim.x) sm[i] = tables[i];
  __syncthreads();
  const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
  for (int64_t qi = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; qi < nq;
       qi += stride) {
    const double x[4] = {q[4 * qi], q[4 * qi + 1], q[4 * qi + 2], q[4 * qi + 3]};
    out[qi] = bspline4d_value(D, sm, coeffs, x);
  }
}

// Surface object with tables uploaded; coefficients are the caller's job.
MangoGpuBSpline4D* new_surface(MangoGpuContext* ctx, const double* grids, const int64_t* sizes) {
  std::vector<double> tab;
  MangoGpuBSpline4D* s = new MangoGpuBSpline4D();
  try {
    s->ctx = ctx;
    bspline_tables(grids, sizes, &s->dims, &tab, &s->knots);
    s->grids.assign(grids, grids + (sizes[0] + sizes[1] + sizes[2] + sizes[3]));
    cudaStream_t st = ctx->stream;
    double* dt = static_cast<double*>(s->d_tables.get(sizeof(double) * tab.size()));
    check(cudaMemcpyAsync(dt, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st), "H2D");
    check(cudaStreamSynchronize(st), "sync");
    int bps = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, bspline4d_eval_kernel, 256,
                                                        sizeof(double) * 4 * s->dims.ktot),
          "occupancy");
    s->blocks = ctx->num_sms * std::max(1, bps);
    return s;
  } catch (...) {
    for (DevBuf* d : {&s->d_tables, &s->d_coeffs}) d->release();
    delete s;
    throw;
  }
}

}  // namespace mgpu

using namespace mgpu;

extern "C" {

MangoStatus mango_gpu_bspline4d_create(MangoGpuContext* ctx, const double* grids,
                                       const int64_t* sizes, const double* coeffs,
                                       MangoGpuBSpline4D** out, MangoError* err) {
  if (!ctx || !grids || !sizes || !coeffs || !out) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  *out = nullptr;
  // BSplineND::create validation (bspline_nd.hpp:70-117)
  int64_t total = 1;
  for (int d = 0; d < 4; ++d) {
    if (sizes[d] < 4 || sizes[d] > kMaxAxis) {
      set_err(err, MANGO_ERR_VALIDATION, "each axis needs 4..512 grid points");
      return MANGO_ERR_VALIDATION;
    }
    total *= sizes[d];
  }
  for (int64_t i = 0; i < total; ++i)
    if (!std::isfinite(coeffs[i])) {
      set_err(err, MANGO_ERR_VALIDATION, "non-finite coefficient");
      return MANGO_ERR_VALIDATION;
    }
  MangoGpuBSpline4D* s = nullptr;
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    s = new_surface(ctx, grids, sizes);
    cudaStream_t st = ctx->stream;
    double* dc = static_cast<double*>(s->d_coeffs.get(sizeof(double) * total));
    check(cudaMemcpyAsync(dc, coeffs, sizeof(double) * total, cudaMemcpyHostToDevice, st), "H2D");
    check(cudaStreamSynchronize(st), "sync");
    *out = s;
    return MANGO_OK;
  } catch (const std::invalid_argument& e) {
    if (s) mango_gpu_bspline4d_destroy(s);
    set_err(err, MANGO_ERR_VALIDATION, e.what());
    return MANGO_ERR_VALIDATION;
  } catch (const std::exception& e) {
    if (s) mango_gpu_bspline4d_destroy(s);
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

void mango_gpu_bspline4d_destroy(MangoGpuBSpline4D* s) {
  if (!s) return;
  cudaSetDevice(s->ctx->device);
  cudaStreamSynchronize(s->ctx->stream);
  for (DevBuf* d : {&s->d_tables, &s->d_coeffs, &s->d_q, &s->d_out}) d->release();
  delete s;
}

MangoStatus mango_gpu_bspline4d_eval_device(MangoGpuBSpline4D* s, const double* d_queries,
                                            uint64_t n, double* d_out, MangoError* err) {
  if (!s || (n > 0 && (!d_queries || !d_out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    const int64_t need = static_cast<int64_t>((n + 255) / 256);
    const int blocks = static_cast<int>(std::min<int64_t>(s->blocks, need));
    bspline4d_eval_kernel<<<blocks, 256, sizeof(double) * 4 * s->dims.ktot, s->ctx->stream>>>(
        s->dims, s->d_tables.as<double>(), s->d_coeffs.as<double>(), d_queries,
        static_cast<int64_t>(n), d_out);
    check(cudaGetLastError(), "bspline4d_eval_kernel launch");
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_bspline4d_eval(MangoGpuBSpline4D* s, const double* queries, uint64_t n,
                                     double* out, MangoError* err) {
  if (!s || (n > 0 && (!queries || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null argument");
    return MANGO_ERR_VALIDATION;
  }
  if (n == 0) return MANGO_OK;
  try {
    check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
    cudaStream_t st = s->ctx->stream;
    double* dq = static_cast<double*>(s->d_q.get(sizeof(double) * 4 * n));
    double* dout = static_cast<double*>(s->d_out.get(sizeof(double) * n));
    check(cudaMemcpyAsync(dq, queries, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, st), "H2D queries");
    MangoStatus rc = mango_gpu_bspline4d_eval_device(s, dq, n, dout, err);
    if (rc != MANGO_OK) return rc;
    check(cudaMemcpyAsync(out, dout, sizeof(double) * n, cudaMemcpyDeviceToHost, st), "D2H");
    check(cudaStreamSynchronize(st), "sync");
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

MangoStatus mango_gpu_bspline4d_knots(const MangoGpuBSpline4D* s, double* out, uint64_t cap,
                                      uint64_t* n_out) {
  if (!s || !n_out) return MANGO_ERR_VALIDATION;
  *n_out = s->knots.size();
  if (out && cap >= s->knots.size()) std::memcpy(out, s->knots.data(), sizeof(double) * s->knots.size());
  return MANGO_OK;
}

MangoStatus mango_gpu_bspline4d_export(const MangoGpuBSpline4D* s, int64_t* sizes, double* grids,
                                       uint64_t grid_cap, double* coeffs, uint64_t coeff_cap,
                                       MangoError* err) {
  if (!s || !sizes) {
    set_err(err, MANGO_ERR_VALIDATION, "null surface or sizes");
    return MANGO_ERR_VALIDATION;
  }
  uint64_t total = 1;
  for (int d = 0; d < 4; ++d) {
    sizes[d] = s->dims.n[d];
    total *= static_cast<uint64_t>(s->dims.n[d]);
  }
  try {
    if (grids) {
      if (grid_cap < s->grids.size()) {
        set_err(err, MANGO_ERR_VALIDATION, "grid buffer too small");
        return MANGO_ERR_VALIDATION;
      }
      std::memcpy(grids, s->grids.data(), sizeof(double) * s->grids.size());
    }
    if (coeffs) {
      if (coeff_cap < total) {
        set_err(err, MANGO_ERR_VALIDATION, "coefficient buffer too small");
        return MANGO_ERR_VALIDATION;
      }
      check(cudaSetDevice(s->ctx->device), "cudaSetDevice");
      check(cudaStreamSynchronize(s->ctx->stream), "sync");
      check(cudaMemcpy(coeffs, s->d_coeffs.p, sizeof(double) * total, cudaMemcpyDeviceToHost), "D2H");
    }
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

}  // extern "C"
