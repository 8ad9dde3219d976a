// fit_host.hpp -- host side of the separable B-spline collocation fit.
//
// One axis of BSplineNDSeparable<double,4>::fit
// (src/math/bspline/bspline_nd_separable.hpp:153-384) solves the same
// collocation system B c = f for every slice along that axis, with
// B[i][j] = N_j(x_i) (BSplineCollocation1D::build_collocation_matrix,
// src/math/bspline/bspline_collocation.hpp:452-480).  The reference factors B
// with LAPACK dgbtrf for every slice; the factors do not depend on the slice,
// so they are computed here once per axis and the device solves every slice
// with them.
#pragma once
#include <cstdint>
#include <vector>

namespace mgpu {

// Collocation matrix of one axis and its banded LU factors (kl = ku = 3,
// partial pivoting; U keeps kl + ku = 6 super-diagonals of fill-in).
struct AxisFactor {
  int n = 0;
  std::vector<double> band;        // n x 4: B[i][col_start[i] + k]
  std::vector<int32_t> col_start;  // first band column of row i
  std::vector<double> lower;       // n x 3: multipliers of column j for rows j+1 .. j+3
  std::vector<int32_t> piv;        // n: row interchanged with row j at step j
  std::vector<double> upper;       // n x 7: U(j, j + d), d = 0 .. 6
  double norm1 = 0.0;              // ||B||_1 (compute_matrix_norm1)
  double cond1 = 0.0;              // ||B||_1 ||B^-1||_1 (inf when singular)
  bool singular = false;
};

// Build and factor the collocation system of the strictly increasing axis
// grid x[0..n), n >= 4.
AxisFactor factor_axis(const double* x, int n);

// Solve B c = f in place with the factors (the device solves the same way).
void solve_axis(const AxisFactor& F, double* c);

}  // namespace mgpu
