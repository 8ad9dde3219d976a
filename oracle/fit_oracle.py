"""CPU restatement of the price-table surface path, for tests only.

TEST INFRASTRUCTURE ONLY: tests/ may import this module as the checker; the
product (mango-option_gb300/) never imports it.

* clamped_knots: clamped_knots_cubic (src/math/bspline/bspline_basis.hpp:47-91)
* basis / collocation_matrix: find_span_cubic + cubic_basis_nonuniform
  (bspline_basis.hpp:120-238) at the grid points, B[i][j] = N_j(x_i)
  (BSplineCollocation1D::build_collocation_matrix,
  src/math/bspline/bspline_collocation.hpp:452-480)
* fit4d: BSplineNDSeparable<double,4>::fit
  (src/math/bspline/bspline_nd_separable.hpp:153-384): axes 3, 2, 1, 0, each
  slice along the axis solved with the axis's collocation matrix.  The
  reference solves with LAPACKE dgbtrf/dgbtrs; this restatement uses numpy's
  dense LU solve, so coefficients agree to the conditioning of B times the
  rounding unit, not bit for bit.  Pinned to the reference's own fit
  (tests/golden/fit.npz) in tests/test_oracle_surface.py.
* european_price / eep_floor / eep_decompose: EuropeanOptionResult::
  compute_price (src/option/european_option.cpp:25-51), eep_floor and
  eep_decompose (src/option/table/eep/eep_decomposer.hpp:21-80).
"""
from __future__ import annotations

import math

import numpy as np

EPS = np.finfo(float).eps


def clamped_knots(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=float)
    n = x.size
    t = np.empty(n + 4)
    t[:4] = x[0]
    if n > 4:
        interior, intervals = n - 4, n - 1
        for idx in range(interior):
            ratio = (idx + 1) / (interior + 1)
            pos = ratio * intervals
            low = min(int(math.floor(pos)), intervals - 1)
            frac = pos - low
            left, right = x[low], x[low + 1]
            knot = (1.0 - frac) * left + frac * right
            eps = max(128.0 * EPS * (right - left), EPS * max(abs(right), 1.0))
            t[4 + idx] = min(max(knot, left + eps), right - eps)
    t[-4:] = x[-1]
    return t


def find_span(t: np.ndarray, x: float) -> int:
    n_ctrl = t.size - 4
    max_span = max(3, n_ctrl - 1)
    if x <= t[3]:
        return 3
    if x >= t[n_ctrl]:
        return max_span
    i = int(np.searchsorted(t[3:n_ctrl + 1], x, side="right")) + 3 - 1
    return min(max(i, 3), max_span)


def basis(t: np.ndarray, i: int, x: float) -> np.ndarray:
    n = t.size
    if abs(x - t[-1]) < 64.0 * EPS * max(abs(t[-1]), 1.0):
        return np.array([1.0, 0.0, 0.0, 0.0])
    prev = np.zeros(4)
    for k in range(4):
        idx = i - k
        if idx >= 0 and idx + 1 < n:
            prev[k] = 1.0 if (t[idx] <= x < t[idx + 1]) else 0.0
    for p in (1, 2, 3):
        cur = np.zeros(4)
        for k in range(4):
            idx = i - k
            if idx >= 0 and idx + p + 1 < n:
                ld, rd = t[idx + p] - t[idx], t[idx + p + 1] - t[idx + 1]
                left = (x - t[idx]) / ld * prev[k] if ld > 0 else 0.0
                right = (t[idx + p + 1] - x) / rd * prev[k - 1] if (rd > 0 and k > 0) else 0.0
                cur[k] = left + right
        prev = cur
    return prev


def collocation_matrix(x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, dtype=float)
    n = x.size
    t = clamped_knots(x)
    B = np.zeros((n, n))
    for i, xi in enumerate(x):
        s = find_span(t, xi)
        N = basis(t, s, xi)
        for k in range(4):
            col = s - k
            if 0 <= col < n:
                B[i, col] = N[k]
    return B


def fit4d(axes, values: np.ndarray) -> np.ndarray:
    c = np.array(values, dtype=float).reshape([a.size for a in axes])
    for ax in (3, 2, 1, 0):
        B = collocation_matrix(axes[ax])
        moved = np.moveaxis(c, ax, 0)
        sol = np.linalg.solve(B, moved.reshape(moved.shape[0], -1))
        c = np.moveaxis(sol.reshape(moved.shape), 0, ax)
    return np.ascontiguousarray(c)


def norm_cdf(x: float) -> float:
    return 0.5 * math.erfc(-x * math.sqrt(0.5))


def european_price(S, K, tau, sigma, r, q, put: bool) -> float:
    if tau <= 0.0 or sigma <= 0.0:
        s, k = S, K
        if tau > 0.0:
            s, k = S * math.exp(-q * tau), K * math.exp(-r * tau)
        return max(k - s, 0.0) if put else max(s - k, 0.0)
    d1 = (math.log(S / K) + (r - q + 0.5 * sigma * sigma) * tau) / (sigma * math.sqrt(tau))
    d2 = d1 - sigma * math.sqrt(tau)
    eq, er = math.exp(-q * tau), math.exp(-r * tau)
    if put:
        return K * er * norm_cdf(-d2) - S * eq * norm_cdf(-d1)
    return S * eq * norm_cdf(d1) - K * er * norm_cdf(d2)


def eep_floor(e: float) -> float:
    if 100.0 * e > 500.0:
        return e
    softplus = math.log1p(math.exp(100.0 * e)) / 100.0
    return max(0.0, softplus - math.log(2.0) / 100.0)


def eep_decompose(axes, tensor: np.ndarray, K_ref: float, q: float, put: bool) -> np.ndarray:
    m, tau, sig, rr = axes
    out = np.array(tensor, dtype=float).reshape(m.size, tau.size, sig.size, rr.size).copy()
    for a in range(m.size):
        spot = math.exp(m[a]) * K_ref
        for b in range(tau.size):
            for c in range(sig.size):
                for d in range(rr.size):
                    eu = european_price(spot, K_ref, tau[b], sig[c], rr[d], q, put)
                    out[a, b, c, d] = eep_floor(K_ref * out[a, b, c, d] - eu)
    return out
