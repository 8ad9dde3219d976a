// bspline.cuh -- 4D cubic B-spline evaluation shared by the query, the
// collocation fit and the price-table surface (bspline.cu, surface.cu).
//
// Restates BSplineND<double,4>::eval (src/math/bspline/bspline_nd.hpp:133-157,
// 314-346) with clamp_bspline_query (bspline_nd.hpp:48-55), find_span_cubic
// (src/math/bspline/bspline_basis.hpp:120-142) and cubic_basis_nonuniform
// (bspline_basis.hpp:164-238).  The span search guarantees
// t_i <= x < t_{i+1}, so the degree-0 basis is (1,0,0,0) and only the
// non-zero entries of the reference's degree-1..3 triangle are evaluated (the
// terms it also computes are exact zeros); Cox-de Boor denominators are
// precomputed reciprocals.  The 256-term tensor product follows the
// reference's nesting and FMA order.
#pragma once
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
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

// clamped_knots_cubic (bspline_basis.hpp:47-91), host.
std::vector<double> clamped_knots(const double* x, int n);

// Packed tables for grids (four axes concatenated, sizes[d] points each):
// knots t, then R1, R2, R3 with R_d[j] = 1 / (t[j+d] - t[j]) (0 where that
// gap is not positive).  Throws std::invalid_argument on a bad axis.
void bspline_tables(const double* grids, const int64_t* sizes, BSplineDims* D,
                    std::vector<double>* tab, std::vector<double>* knots);

// BSplineND<double,4>::eval at x[0..3] (DAX < 0), or eval_partial along
// axis DAX (bspline_nd.hpp:168-199: the derivative basis
// cubic_basis_derivative_nonuniform, bspline_basis.hpp:258-330, on that axis,
// without the right-end special case); sm holds the packed tables.
// DAX >= 0: the derivative basis of order ORD (1: cubic_basis_derivative_
// nonuniform, 2: cubic_basis_second_derivative_nonuniform, bspline_basis.hpp:
// 343-410) on that axis, the value basis on the others.
template <int DAX = -1, int ORD = 1>
__device__ __forceinline__ double bspline4d_eval_t(const BSplineDims& D, const double* sm,
                                                   const double* __restrict__ coeffs,
                                                   const double* xq) {
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
    double x = xq[d];
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
    if (d == DAX && ORD == 2) {
      // degree-1 basis, its derivative quadratics, then the cubic's second
      // derivative (zero-length knot spans give zero reciprocals)
      const double n10 = (x - t[i]) * R1[i];
      const double n11 = (t[i + 1] - x) * R1[i];
      const double q0 = 2.0 * R2[i] * n10;
      const double q1 = 2.0 * R2[i - 1] * n11 - 2.0 * R2[i] * n10;
      const double q2 = 0.0 - 2.0 * R2[i - 1] * n11;
      w[d][0] = 3.0 * R3[i] * q0;
      w[d][1] = 3.0 * R3[i - 1] * q1 - 3.0 * R3[i] * q0;
      w[d][2] = 3.0 * R3[i - 2] * q2 - 3.0 * R3[i - 1] * q1;
      w[d][3] = 0.0 - 3.0 * R3[i - 2] * q2;
      continue;
    }
    if (d == DAX) {
      const double n10 = (x - t[i]) * R1[i];
      const double n11 = (t[i + 1] - x) * R1[i];
      const double n20 = (x - t[i]) * R2[i] * n10;
      const double n21 = (x - t[i - 1]) * R2[i - 1] * n11 + (t[i + 2] - x) * R2[i] * n10;
      const double n22 = (t[i + 1] - x) * R2[i - 1] * n11;
      w[d][0] = 3.0 * R3[i] * n20;
      w[d][1] = 3.0 * R3[i - 1] * n21 - 3.0 * R3[i] * n20;
      w[d][2] = 3.0 * R3[i - 2] * n22 - 3.0 * R3[i - 1] * n21;
      w[d][3] = 0.0 - 3.0 * R3[i - 2] * n22;
      continue;
    }
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
  return s0;
}

__device__ __forceinline__ double bspline4d_value(const BSplineDims& D, const double* sm,
                                                  const double* __restrict__ coeffs,
                                                  const double* xq) {
  return bspline4d_eval_t<-1>(D, sm, coeffs, xq);
}

}  // namespace mgpu

// A device-resident 4D surface: packed knot tables and coefficients.
struct MangoGpuBSpline4D {
  MangoGpuContext* ctx = nullptr;
  mgpu::BSplineDims dims{};
  mgpu::DevBuf d_tables, d_coeffs, d_q, d_out;
  std::vector<double> knots;  // packed, for inspection
  std::vector<double> grids;  // packed axes, for export
  int blocks = 0;
};
