// fit_host.cpp -- collocation matrix and banded LU of one fit axis.
//
// The basis restates cubic_basis_nonuniform and find_span_cubic
// (src/math/bspline/bspline_basis.hpp:120-238) with the reference's divides
// and order (compiled with -ffp-contract=off); the knots are
// clamped_knots_cubic (bspline_basis.hpp:47-91).  The factorisation follows
// the published LAPACK band LU (dgbtf2: partial pivoting over the kl rows
// below the diagonal, the pivot column scaled by the reciprocal of the pivot,
// rank-1 update of the band to its right, row interchanges applied to the
// columns from the pivot on) and the solve follows dgbtrs + dtbsv (forward
// elimination with the interchanges, then column-oriented back substitution
// with a divide by each diagonal entry).  LAPACKE itself is not available in
// this build; the reference links the system library there.
#include "fit_host.hpp"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <limits>

namespace mgpu {

std::vector<double> clamped_knots(const double* x, int n);  // bspline.cu

namespace {

int find_span(const std::vector<double>& t, double x) {
  const int n_ctrl = static_cast<int>(t.size()) - 4;
  const int max_span = std::max(3, n_ctrl - 1);
  if (x <= t[3]) return 3;
  if (x >= t[n_ctrl]) return max_span;
  const auto it = std::upper_bound(t.begin() + 3, t.begin() + n_ctrl + 1, x);
  const int i = static_cast<int>(it - t.begin()) - 1;
  return std::clamp(i, 3, max_span);
}

void basis(const std::vector<double>& t, int i, double x, double N[4]) {
  const int n = static_cast<int>(t.size());
  if (std::fabs(x - t.back()) < 64.0 * DBL_EPSILON * std::max(std::fabs(t.back()), 1.0)) {
    N[0] = 1.0;
    N[1] = N[2] = N[3] = 0.0;
    return;
  }
  double N0[4] = {0, 0, 0, 0}, N1[4] = {0, 0, 0, 0}, N2[4] = {0, 0, 0, 0};
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 1 < n) N0[k] = (t[idx] <= x && x < t[idx + 1]) ? 1.0 : 0.0;
  }
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 2 < n) {
      const double ld = t[idx + 1] - t[idx], rd = t[idx + 2] - t[idx + 1];
      const double left = ld > 0.0 ? (x - t[idx]) / ld * N0[k] : 0.0;
      const double right = (rd > 0.0 && k > 0) ? (t[idx + 2] - x) / rd * N0[k - 1] : 0.0;
      N1[k] = left + right;
    }
  }
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 3 < n) {
      const double ld = t[idx + 2] - t[idx], rd = t[idx + 3] - t[idx + 1];
      const double left = ld > 0.0 ? (x - t[idx]) / ld * N1[k] : 0.0;
      const double right = (rd > 0.0 && k > 0) ? (t[idx + 3] - x) / rd * N1[k - 1] : 0.0;
      N2[k] = left + right;
    }
  }
  for (int k = 0; k < 4; ++k) {
    const int idx = i - k;
    if (idx >= 0 && idx + 4 < n) {
      const double ld = t[idx + 3] - t[idx], rd = t[idx + 4] - t[idx + 1];
      const double left = ld > 0.0 ? (x - t[idx]) / ld * N2[k] : 0.0;
      const double right = (rd > 0.0 && k > 0) ? (t[idx + 4] - x) / rd * N2[k - 1] : 0.0;
      N[k] = left + right;
    } else {
      N[k] = 0.0;
    }
  }
}

}  // namespace

AxisFactor factor_axis(const double* x, int n) {
  AxisFactor F;
  F.n = n;
  const std::vector<double> t = clamped_knots(x, n);
  // Dense B (n is at most a few hundred), then its band rows.
  std::vector<double> A(static_cast<size_t>(n) * n, 0.0);
  auto a = [&](int r, int c) -> double& { return A[static_cast<size_t>(r) * n + c]; };
  F.band.assign(static_cast<size_t>(n) * 4, 0.0);
  F.col_start.assign(static_cast<size_t>(n), 0);
  for (int i = 0; i < n; ++i) {
    const int span = find_span(t, x[i]);
    double N[4];
    basis(t, span, x[i], N);
    const int cs = std::max(0, span - 3);
    F.col_start[i] = cs;
    for (int k = 0; k < 4; ++k) {
      const int col = span - k;
      if (col >= 0 && col < n && col - cs >= 0 && col - cs < 4) {
        F.band[static_cast<size_t>(i) * 4 + (col - cs)] = N[k];
        a(i, col) = N[k];
      }
    }
  }
  // compute_matrix_norm1: largest absolute column sum.
  for (int c = 0; c < n; ++c) {
    double s = 0.0;
    for (int r = 0; r < n; ++r) s += std::fabs(a(r, c));
    F.norm1 = std::max(F.norm1, s);
  }
  // Band LU with partial pivoting (dgbtf2 order).
  constexpr int kl = 3, ku = 3;
  F.lower.assign(static_cast<size_t>(n) * kl, 0.0);
  F.piv.assign(static_cast<size_t>(n), 0);
  F.upper.assign(static_cast<size_t>(n) * (kl + ku + 1), 0.0);
  for (int j = 0; j < n; ++j) {
    const int km = std::min(kl, n - 1 - j);
    int p = j;
    double amax = std::fabs(a(j, j));
    for (int r = j + 1; r <= j + km; ++r)
      if (std::fabs(a(r, j)) > amax) {
        amax = std::fabs(a(r, j));
        p = r;
      }
    F.piv[j] = p;
    if (a(p, j) == 0.0) {
      F.singular = true;
      continue;
    }
    const int cend = std::min(n - 1, j + kl + ku);
    if (p != j)
      for (int c = j; c <= cend; ++c) std::swap(a(p, c), a(j, c));
    const double rp = 1.0 / a(j, j);
    for (int r = j + 1; r <= j + km; ++r) a(r, j) *= rp;
    for (int c = j + 1; c <= cend; ++c) {
      const double u = a(j, c);
      if (u == 0.0) continue;
      for (int r = j + 1; r <= j + km; ++r) a(r, c) = a(r, c) + a(r, j) * (-u);
    }
    for (int r = j + 1; r <= j + km; ++r) F.lower[static_cast<size_t>(j) * kl + (r - j - 1)] = a(r, j);
  }
  for (int j = 0; j < n; ++j)
    for (int d = 0; d <= kl + ku && j + d < n; ++d)
      F.upper[static_cast<size_t>(j) * (kl + ku + 1) + d] = a(j, j + d);
  // ||B^-1||_1 from the factors, column by column.
  if (F.singular) {
    F.cond1 = std::numeric_limits<double>::infinity();
  } else {
    double inv_norm = 0.0;
    std::vector<double> e(static_cast<size_t>(n));
    for (int c = 0; c < n; ++c) {
      std::fill(e.begin(), e.end(), 0.0);
      e[c] = 1.0;
      solve_axis(F, e.data());
      double s = 0.0;
      for (int r = 0; r < n; ++r) s += std::fabs(e[r]);
      inv_norm = std::max(inv_norm, s);
    }
    F.cond1 = F.norm1 * inv_norm;
  }
  return F;
}

void solve_axis(const AxisFactor& F, double* c) {
  const int n = F.n;
  for (int j = 0; j + 1 < n; ++j) {
    const int p = F.piv[j];
    if (p != j) std::swap(c[p], c[j]);
    const double bj = -c[j];
    const int lm = std::min(3, n - 1 - j);
    for (int i = 1; i <= lm; ++i) c[j + i] = c[j + i] + F.lower[static_cast<size_t>(j) * 3 + i - 1] * bj;
  }
  for (int j = n - 1; j >= 0; --j) {
    if (c[j] == 0.0) continue;
    c[j] = c[j] / F.upper[static_cast<size_t>(j) * 7];
    const double tmp = c[j];
    for (int i = j - 1; i >= std::max(0, j - 6); --i)
      c[i] = c[i] - tmp * F.upper[static_cast<size_t>(i) * 7 + (j - i)];
  }
}

}  // namespace mgpu
