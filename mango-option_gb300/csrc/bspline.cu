// bspline.cu -- 4D cubic B-spline surface query on the GPU.
//
// Restates BSplineND<double,4>::eval (src/math/bspline/bspline_nd.hpp:133-157,
// 314-346) with clamp_bspline_query (bspline_nd.hpp:48-55), find_span_cubic
// (src/math/bspline/bspline_basis.hpp:120-142) and cubic_basis_nonuniform
// (bspline_basis.hpp:164-238); knots from clamped_knots_cubic
// (bspline_basis.hpp:47-91).
//
// GB300 design: one thread per query, FP64 throughout.  Knots and the
// reciprocals of every Cox-de Boor denominator live in shared memory, so the
// basis needs no divide.  The span search guarantees t_i <= x < t_{i+1}, so
// the degree-0 basis is (1,0,0,0) and only the non-zero entries of the
// reference's degree-1..3 triangle are evaluated (the terms it also
// computes are exact zeros).  The 256-term tensor product follows the
// reference's nesting and FMA order; the coefficient table (2.4 MB at
// 50x30x20x10) stays in L2 and is read through the read-only path.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "engine.hpp"

namespace mgpu {

constexpr int kMaxAxis = 512;  // grid points per axis (knots = points + 4)

struct BSplineDims {
  int n[4];      // grid points per axis
  int koff[4];   // offset of each axis's knots in the packed knot array
  int ktot;      // total knots
  double lo[4];  // grid front
  double hi[4];  // grid back
  double hi_below[4];  // nextafter(hi, -inf)
  double tlast[4];     // knots.back()
};

namespace {

// clamped_knots_cubic (bspline_basis.hpp:47-91).
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

}  // namespace

// Packed per-axis tables in shared memory: knots t, then R1, R2, R3 with
// R_d[j] = 1 / (t[j+d] - t[j]) (0 where that gap is not positive).
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
    int span[4];
    double w[4][4];
#pragma unroll
    for (int d = 0; d < 4; ++d) {
      const double* t = sm + D.koff[d];
      const double* R1 = t + D.ktot;
      const double* R2 = R1 + D.ktot;
      const double* R3 = R2 + D.ktot;
      const int nk = D.n[d] + 4;
      // clamp_bspline_query
      double x = q[4 * qi + d];
      if (x <= D.lo[d]) x = D.lo[d];
      else if (x >= D.hi[d]) x = D.hi_below[d];
      // find_span_cubic: upper_bound over t[3 .. n_ctrl]
      const int n_ctrl = nk - 4;
      const int max_span = max(3, n_ctrl - 1);
      int i;
      if (x <= t[3]) {
        i = 3;
      } else if (x >= t[n_ctrl]) {
        i = max_span;
      } else {
        int lo = 3, hi = n_ctrl + 1;  // first index with t[idx] > x
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (t[mid] <= x) lo = mid + 1; else hi = mid;
        }
        i = min(max(lo - 1, 3), max_span);
      }
      span[d] = i;
      // cubic_basis_nonuniform
      if (fabs(x - D.tlast[d]) < 64.0 * DBL_EPSILON * fmax(fabs(D.tlast[d]), 1.0)) {
        w[d][0] = 1.0;
        w[d][1] = 0.0;
        w[d][2] = 0.0;
        w[d][3] = 0.0;
      } else {
        const double n10 = (x - t[i]) * R1[i];
        const double n11 = (t[i + 1] - x) * R1[i];
        const double n20 = (x - t[i]) * R2[i] * n10;
        const double n21 = (x - t[i - 1]) * R2[i - 1] * n11 + (t[i + 2] - x) * R2[i] * n10;
        const double n22 = (t[i + 1] - x) * R2[i - 1] * n11;
        w[d][0] = (x - t[i]) * R3[i] * n20;
        w[d][1] = (x - t[i - 1]) * R3[i - 1] * n21 + (t[i + 3] - x) * R3[i] * n20;
        w[d][2] = (x - t[i - 2]) * R3[i - 2] * n22 + (t[i + 2] - x) * R3[i - 1] * n21;
        w[d][3] = (t[i + 1] - x) * R3[i - 2] * n22;
      }
    }
    // eval_tensor_product (bspline_nd.hpp:314-346)
    const int d1 = D.n[1], d2 = D.n[2], d3 = D.n[3];
    double s0 = 0.0;
#pragma unroll
    for (int o0 = 0; o0 < 4; ++o0) {
      const int i0 = span[0] - o0;
      if (static_cast<unsigned>(i0) >= static_cast<unsigned>(D.n[0])) continue;
      double s1 = 0.0;
#pragma unroll
      for (int o1 = 0; o1 < 4; ++o1) {
        const int i1 = span[1] - o1;
        if (static_cast<unsigned>(i1) >= static_cast<unsigned>(d1)) continue;
        double s2 = 0.0;
#pragma unroll
        for (int o2 = 0; o2 < 4; ++o2) {
          const int i2 = span[2] - o2;
          if (static_cast<unsigned>(i2) >= static_cast<unsigned>(d2)) continue;
          const double* c = coeffs + (static_cast<size_t>(i0 * d1 + i1) * d2 + i2) * d3;
          double s3 = 0.0;
#pragma unroll
          for (int o3 = 0; o3 < 4; ++o3) {
            const int i3 = span[3] - o3;
            if (static_cast<unsigned>(i3) >= static_cast<unsigned>(d3)) continue;
            s3 = fma(__ldg(c + i3), w[3][o3], s3);
          }
          s2 = fma(s3, w[2][o2], s2);
        }
        s1 = fma(s2, w[1][o1], s1);
      }
      s0 = fma(s1, w[0][o0], s0);
    }
    out[qi] = s0;
  }
}

}  // namespace mgpu

struct MangoGpuBSpline4D {
  MangoGpuContext* ctx = nullptr;
  mgpu::BSplineDims dims{};
  mgpu::DevBuf d_tables, d_coeffs, d_q, d_out;
  std::vector<double> knots;  // packed, for inspection
  int blocks = 0;
};

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
    s = new MangoGpuBSpline4D();
    s->ctx = ctx;
    BSplineDims& D = s->dims;
    int koff = 0;
    const double* g = grids;
    std::vector<std::vector<double>> kn(4);
    for (int d = 0; d < 4; ++d) {
      const int n = static_cast<int>(sizes[d]);
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
    std::vector<double> tab(static_cast<size_t>(4 * koff), 0.0);
    for (int d = 0; d < 4; ++d) {
      const std::vector<double>& t = kn[d];
      const int nk = static_cast<int>(t.size());
      for (int j = 0; j < nk; ++j) {
        tab[D.koff[d] + j] = t[j];
        s->knots.push_back(t[j]);
        for (int deg = 1; deg <= 3; ++deg) {
          double r = 0.0;
          if (j + deg < nk) {
            const double den = t[j + deg] - t[j];
            if (den > 0.0) r = 1.0 / den;
          }
          tab[static_cast<size_t>(deg) * koff + D.koff[d] + j] = r;
        }
      }
    }
    cudaStream_t st = ctx->stream;
    double* dt = static_cast<double*>(s->d_tables.get(sizeof(double) * tab.size()));
    double* dc = static_cast<double*>(s->d_coeffs.get(sizeof(double) * total));
    check(cudaMemcpyAsync(dt, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st), "H2D");
    check(cudaMemcpyAsync(dc, coeffs, sizeof(double) * total, cudaMemcpyHostToDevice, st), "H2D");
    check(cudaStreamSynchronize(st), "sync");
    int bps = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, bspline4d_eval_kernel, 256,
                                                        sizeof(double) * 4 * koff),
          "occupancy");
    s->blocks = ctx->num_sms * std::max(1, bps);
    *out = s;
    return MANGO_OK;
  } catch (const std::exception& e) {
    delete s;
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

}  // extern "C"
