// march_tan.cu -- the cached-factorisation American march with forward-mode
// tangents: value, delta and the exact discrete derivatives of the price
// along volatility (and, for the Greeks, rate and dividend yield) in one
// sweep of the primal.
//
// The primal is march.cu's march, bit for bit in its arithmetic: the
// reference's PDESolver::solve with the Rannacher start and TR-BDF2 stages
// (src/pde/internal/pde_solver.hpp:114-178, 342-447), the projected stage
// with the deep-ITM lock (pde_solver.hpp:525-729) and solve_thomas_projected
// (src/math/thomas_solver.hpp:321-420) on cached, time-invariant stage
// factorisations.  Beside it every lane carries ND tangents through the same
// operations, so the derivative is that of the discrete price the march
// computes (the quantity central differences on the same grid approximate):
//  * the operator's coefficients a = sigma^2/2, b = r - q - a, c = -r enter
//    the Jacobian rows linearly, so a direction's row derivative is
//    da * D2 + db * D1 + dc * I with D2, D1 the grid's second- and
//    first-difference stencils (assemble_jacobian form,
//    spatial_operator.hpp:123-163);
//  * the cached row factors (pre-scaled stencil, -l/pivot, -c', the stage-2
//    weights over the pivot) are differentiated once per option in
//    prep_tan_kernel, along the unlocked factor recurrence, so a cached row
//    costs the primal's 4 + 1 + 3 + 1 FMAs plus 8 + 2 + 6 + 2 per direction;
//  * rows off the cache (a locked row and the rows after it until the
//    recomputed factor is bit-identical to the cached one) differentiate the
//    reference's recurrence itself: denominator, reciprocal, c' and d';
//  * the projected back substitution x_i = max(y_i, psi_i) passes the
//    tangent of y_i unless y_i < psi_i (the obstacle binds; psi does not
//    depend on the parameters), and a locked row (identity, rhs psi) has a
//    zero tangent;
//  * Dirichlet rows carry the derivative of their boundary value: zero, except
//    the call's right boundary e^x - e^{-r t} along the rate (t e^{-r t}).
// The functionals follow AmericanOptionResult (american_option_result.cpp:
// 25-60): the natural spline is linear in its data, so dV/dtheta = K times
// the spline of the tangent at ln(S/K) (zero where max(0, .) clamps), and
// dV/dK = S(x) - S'(x) because the log-moneyness grid does not depend on K.
//
// GB300 layout: as march.cu -- one warp per tile of 32 options, one lane per
// option, rows [row][array][lane]; the tangent arrays of a tile live in a
// second pool with the same row order ([row][direction][array][lane]) so a
// warp's accesses coalesce.  Each sweep streams its row inputs through a
// per-warp shared-memory ring filled by cp.async, kTanAhead rows ahead of
// the row being solved.  FP64 issue and HBM streaming bound the kernel; no
// tensor cores (nothing here is a contraction).
#include "march_dev.cuh"

#include <cuda_runtime.h>
#include <climits>
#include <type_traits>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "engine.hpp"
#include "march_tan.cuh"

namespace mgpu {

namespace {

// Parameter derivatives of (hss = a, drift = b, rate = -c) per direction.
struct Dir {
  double dh, dd, dr;
};

template <int ND>
__device__ __forceinline__ void directions(const int32_t* dirs, double sigma, Dir* d) {
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    const int k = dirs[j];
    if (k == kDirSigma) d[j] = Dir{sigma, -sigma, 0.0};  // d/dsigma: da = sigma, db = -sigma
    else if (k == kDirRate) d[j] = Dir{0.0, 1.0, 1.0};   // d/dr: db = 1, dc = -1
    else d[j] = Dir{0.0, -1.0, 0.0};                     // d/dq: db = -1
  }
}

}  // namespace

// ------------------------------------------------------------- tangent prep --
// One lane per option, after prep_kernel: the derivative of every cached row
// factor along each direction, the operator's row derivative for rows off the
// cache, and the zero initial tangent (u^0 = payoff).
template <int ND>
__device__ __forceinline__ void prep_tan_body(const TileDev* __restrict__ tiles, int ntiles,
                                const OptDev* __restrict__ opts, const double* __restrict__ xs,
                                const double* __restrict__ pool, double* __restrict__ tpool,
                                TanConst tc, MarchConst mc) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = gt / kTile, lane = gt % kTile;
  if (t >= ntiles) return;
  const TileDev td = tiles[t];
  if (lane >= td.count) return;
  const int k = td.first + lane;
  if ((mc.active && !mc.active[k]) || k >= mc.tv_first) return;
  const OptDev o = opts[k];
  const int n = o.n;
  const TileView V{const_cast<double*>(pool) + td.off + lane, td.nx};
  const TanView<ND> W{tpool + tan_off<ND>(td) + lane};
  const double* X = xs + td.xoff + lane;
  auto x = [&](int i) { return X[static_cast<size_t>(i) * kTile]; };
  const double sigma = mc.sigma ? mc.sigma[k] : o.sigma;
  Dir dir[ND];
  directions<ND>(tc.dirs, sigma, dir);
  const double dt = o.dt;
  const double w1 = mc.gamma * dt / 2.0;
  const double w2 = (1.0 - mc.gamma) * dt / (2.0 - mc.gamma);

#pragma unroll
  for (int j = 0; j < ND; ++j)
    for (int i = 0; i < n; ++i) {
      W.at(j, T_U, i) = 0.0;
      W.at(j, T_G, i) = 0.0;
    }
  double cp1 = 0.0, cp2 = 0.0;
  double tcp1[ND], tcp2[ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) tcp1[j] = tcp2[j] = 0.0;
  for (int i = 1; i < n - 1; ++i) {
    const double dxl = x(i) - x(i - 1), dxr = x(i + 1) - x(i);
    const double dxa = (dxl + dxr) / 2.0;
    const double d1d = dxl + dxr;
    // assemble_jacobian's stencils per unit coefficient
    const double s2l = 1.0 / (dxl * dxa), s2d = -(1.0 / dxl + 1.0 / dxr) / dxa,
                 s2u = 1.0 / (dxr * dxa);
    const double s1l = -dxr / (dxl * d1d), s1d = (dxr - dxl) / (dxl * dxr),
                 s1u = dxl / (dxr * d1d);
    const double* r = V.rp(i);
    const double l1 = r[A_L1 * kTile], dg1 = r[A_D1 * kTile], u1 = r[A_U1 * kTile];
    const double l2 = r[A_L2 * kTile], dg2 = r[A_D2 * kTile], u2 = r[A_U2 * kTile];
    const double el = r[A_E1L0 * kTile], ed = r[A_E1D0 * kTile], eu = r[A_E1U0 * kTile];
    // the same recurrence as prep_kernel, so inv1 / inv2 are its values
    const double inv1 = 1.0 / fma(-l1, cp1, dg1);
    const double inv2 = 1.0 / fma(-l2, cp2, dg2);
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const double jl = dir[j].dh * s2l + dir[j].dd * s1l;
      const double jd = dir[j].dh * s2d + dir[j].dd * s1d - dir[j].dr;
      const double ju = dir[j].dh * s2u + dir[j].dd * s1u;
      W.at(j, T_JL, i) = jl;
      W.at(j, T_JD, i) = jd;
      W.at(j, T_JU, i) = ju;
      // stage 1: bands -w1 J, explicit stencil (I + w1 L) -> derivative w1 J'
      {
        const double tl = -w1 * jl, tdg = -w1 * jd, tu = -w1 * ju;
        const double tden = tdg - tl * cp1 - l1 * tcp1[j];
        const double tinv = -(inv1 * inv1) * tden;
        const double tcp = tu * inv1 + u1 * tinv;
        W.at(j, T_E1L, i) = (w1 * jl) * inv1 + el * tinv;
        W.at(j, T_E1D, i) = (w1 * jd) * inv1 + ed * tinv;
        W.at(j, T_E1U, i) = (w1 * ju) * inv1 + eu * tinv;
        W.at(j, T_N1H, i) = -(tl * inv1 + l1 * tinv);
        W.at(j, T_NC1, i) = -tcp;
        tcp1[j] = tcp;
      }
      // stage 2: bands -w2 J, rhs alpha g + beta u
      {
        const double tl = -w2 * jl, tdg = -w2 * jd, tu = -w2 * ju;
        const double tden = tdg - tl * cp2 - l2 * tcp2[j];
        const double tinv = -(inv2 * inv2) * tden;
        const double tcp = tu * inv2 + u2 * tinv;
        W.at(j, T_A2H, i) = mc.alpha * tinv;
        W.at(j, T_B2H, i) = mc.beta * tinv;
        W.at(j, T_N2H, i) = -(tl * inv2 + l2 * tinv);
        W.at(j, T_NC2, i) = -tcp;
        tcp2[j] = tcp;
      }
    }
    cp1 = u1 * inv1;
    cp2 = u2 * inv2;
  }
}

// ------------------------------------------------------------ tangent march --

namespace {

enum StageKind { kRannacher = 0, kStage1 = 1, kStage2 = 2 };

template <int ND>
struct TanRing {
  static constexpr int kAhead = ND == 1 ? 4 : 2;   // rows in flight
  static constexpr int kSlots = kAhead + 1;        // a slot is refilled one row after it was read
  static constexpr int kArrays = 6 + 5 * ND;       // per row: primal 5, per direction 5, psi
  static constexpr int kPsi = 5 + 5 * ND;          // the lock test's obstacle
  static constexpr int kSlot = kArrays * kTile;    // doubles per slot
  static constexpr int kWarp = kSlots * kSlot;     // doubles per warp
};

__device__ __forceinline__ void cp_async8(double* sdst, const double* gsrc) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(sdst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// y < psi for psi >= +0, on the bit patterns (a negative y always binds).
__device__ __forceinline__ bool binds(double y, double psi) {
  return __double_as_longlong(y) < __double_as_longlong(psi);
}

template <int ND>
struct TanVec {
  double v[ND];
};

// Forward-sweep inputs of row i into ring slot i % kSlots: the primal's five,
// then per direction its four row-factor derivatives and its state.
template <int K, int ND>
__device__ __forceinline__ void issue_fwd_t(const TileView& V, const TanView<ND>& W, double* R,
                                            int a_in, int t_in, int i, int flo, int fhi) {
  using RG = TanRing<ND>;
  double* s = R + (i % RG::kSlots) * RG::kSlot;
  const double* p = V.rp(i);
  if (i >= flo && i <= fhi) cp_async8(s + RG::kPsi * kTile, p + A_PSI * kTile);
  if (K == kStage1) {
    cp_async8(s, p + A_E1L * kTile);
    cp_async8(s + kTile, p + A_E1D * kTile);
    cp_async8(s + 2 * kTile, p + A_E1U * kTile);
    cp_async8(s + 3 * kTile, p + A_N1H * kTile);
    cp_async8(s + 4 * kTile, V.rp(i + 1) + A_U * kTile);
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      double* q = s + (5 + 5 * j) * kTile;
      cp_async8(q, &W.at(j, T_E1L, i));
      cp_async8(q + kTile, &W.at(j, T_E1D, i));
      cp_async8(q + 2 * kTile, &W.at(j, T_E1U, i));
      cp_async8(q + 3 * kTile, &W.at(j, T_N1H, i));
      cp_async8(q + 4 * kTile, &W.at(j, T_U, i + 1));
    }
  } else if (K == kStage2) {
    cp_async8(s, p + A_A2H * kTile);
    cp_async8(s + kTile, p + A_B2H * kTile);
    cp_async8(s + 2 * kTile, p + A_N2H * kTile);
    cp_async8(s + 3 * kTile, p + A_G * kTile);
    cp_async8(s + 4 * kTile, p + A_U * kTile);
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      double* q = s + (5 + 5 * j) * kTile;
      cp_async8(q, &W.at(j, T_A2H, i));
      cp_async8(q + kTile, &W.at(j, T_B2H, i));
      cp_async8(q + 2 * kTile, &W.at(j, T_N2H, i));
      cp_async8(q + 3 * kTile, &W.at(j, T_G, i));
      cp_async8(q + 4 * kTile, &W.at(j, T_U, i));
    }
  } else {
    cp_async8(s + 3 * kTile, p + a_in * kTile);
#pragma unroll
    for (int j = 0; j < ND; ++j) cp_async8(s + (5 + 5 * j + 3) * kTile, &W.at(j, t_in, i));
  }
}

// Back-substitution inputs of row i: -c', psi, d', then per direction the
// -c' derivative and the tangent d'.  For the rows [lo, hi] this sweep solved
// off the cache, -c' and its derivatives are the sweep's own (A_CP, T_CP)
// rather than the cached ones.
template <int K, int ND>
__device__ __forceinline__ void issue_bwd_t(const TileView& V, const TanView<ND>& W, double* R,
                                            int i, int lo, int hi) {
  using RG = TanRing<ND>;
  double* s = R + (i % RG::kSlots) * RG::kSlot;
  const double* p = V.rp(i);
  const bool off = i >= lo && i <= hi;
  cp_async8(s, p + (off ? A_CP : (K == kStage2 ? A_NC2 : A_NC1)) * kTile);
  cp_async8(s + kTile, p + A_PSI * kTile);
  cp_async8(s + 2 * kTile, p + A_D * kTile);
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    cp_async8(s + (3 + 2 * j) * kTile, &W.at(j, off ? T_CP : (K == kStage2 ? T_NC2 : T_NC1), i));
    cp_async8(s + (4 + 2 * j) * kTile, &W.at(j, T_D, i));
  }
}

// One implicit stage with its tangents, for one lane
// (solve_implicit_stage_projected, pde_solver.hpp:525-729):
//   kRannacher: rhs = guess = u_prev (a_in / t_in), bands LR/DR/UR, never cached.
//   kStage1:    rhs = u + w1 L(u) of u^n (A_U / T_U), writes A_G / T_G.
//   kStage2:    rhs = alpha g + beta u^n (g = A_G / T_G), writes a_out / t_out.
// wst is the stage's weight (bands = I - wst J); tbcr the tangent of the
// right boundary value.  Lanes that are not live execute no memory operation.
template <int K, int ND>
__device__ __noinline__ int32_t stage_t(bool live, int n, const TileView V, const TanView<ND> W,
                                        const uint8_t* __restrict__ F, bool nocache, double bcl,
                                        double bcr, TanVec<ND> tbcr, double alpha, double beta,
                                        double wst, int a_in, int a_out, int t_in, int t_out,
                                        int32_t st, int flo, int fhi, double* R, int cflo,
                                        int cfhi, bool cexact) {
  using RG = TanRing<ND>;
  constexpr int aL = (K == kRannacher) ? A_LR : (K == kStage1 ? A_L1 : A_L2);
  constexpr int aDg = (K == kRannacher) ? A_DR : (K == kStage1 ? A_D1 : A_D2);
  constexpr int aU = (K == kRannacher) ? A_UR : (K == kStage1 ? A_U1 : A_U2);
  constexpr int aNC = (K == kStage2) ? A_NC2 : A_NC1;
  constexpr int tNC = (K == kStage2) ? T_NC2 : T_NC1;
  const int last = V.NX - 2;
  const bool always_fresh = (K == kRannacher) || nocache;
  R += threadIdx.x & (kTile - 1);
  __threadfence_block();

  // ---- forward elimination
  double dprev = bcl, cprev = 0.0;
  double tdprev[ND], tcprev[ND], tum[ND], tu0[ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) tdprev[j] = tcprev[j] = tum[j] = tu0[j] = 0.0;
  bool fresh = always_fresh;
  int lo = INT_MAX, hi = -1;
  double um = 0.0, u0 = 0.0;
  if (K == kStage1 && live) {
    um = V.at(A_U, 0);
    u0 = V.at(A_U, 1);
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      tum[j] = W.at(j, T_U, 0);
      tu0[j] = W.at(j, T_U, 1);
    }
  }
  const int stop = live ? min(last, n - 2) : 0;
  for (int j = 1; j <= RG::kAhead; ++j) {
    if (j <= stop) issue_fwd_t<K, ND>(V, W, R, a_in, t_in, j, flo, fhi);
    cp_commit();
  }
  auto row = [&](int i, auto may_lock) {
    cp_wait<RG::kAhead - 1>();
    const double* s = R + (i % RG::kSlots) * RG::kSlot;
    double ra = 0.0, rb = 0.0, rc, rnl = 0.0, rv = 0.0;
    if (K != kRannacher) {
      ra = s[0];
      rb = s[kTile];
      rnl = s[(K == kStage1 ? 3 : 2) * kTile];
      rv = s[4 * kTile];
    }
    rc = s[(K == kStage1 ? 2 : 3) * kTile];
    double qa[ND], qb[ND], qc[ND], qn[ND], qv[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const double* q = s + (5 + 5 * j) * kTile;
      qa[j] = q[0];
      qb[j] = q[kTile];
      qc[j] = q[2 * kTile];
      qn[j] = q[3 * kTile];
      qv[j] = q[4 * kTile];
    }
    if (i + RG::kAhead <= stop) issue_fwd_t<K, ND>(V, W, R, a_in, t_in, i + RG::kAhead, flo, fhi);
    cp_commit();
    const double g = (K == kStage1) ? u0 : rc;
    bool lock = false;
    double psi_i = 0.0;
    // this lane's candidate rows: its own contiguous block, else the flags
    if (decltype(may_lock)::value && (cexact ? (i >= cflo && i <= cfhi) : ROW(F, i) != 0)) {
      psi_i = s[RG::kPsi * kTile];
      lock = (g - psi_i < 1e-8);
    }
    double dcur, tdcur[ND];
    if (!lock && !fresh) {
      if (K == kStage1) {
        dcur = fma(rnl, dprev, fma(ra, um, fma(rb, u0, rc * rv)));
#pragma unroll
        for (int j = 0; j < ND; ++j)
          tdcur[j] = fma(rnl, tdprev[j],
                         fma(ra, tum[j],
                             fma(rb, tu0[j],
                                 fma(rc, qv[j],
                                     fma(qa[j], um, fma(qb[j], u0, fma(qc[j], rv, qn[j] * dprev)))))));
      } else {
        // slot per direction: d(a2h), d(b2h), d(n2h), tangent of g, tangent of u
        dcur = fma(rnl, dprev, fma(ra, g, rb * rv));
#pragma unroll
        for (int j = 0; j < ND; ++j)
          tdcur[j] = fma(rnl, tdprev[j],
                         fma(ra, qn[j], fma(rb, qv[j], fma(qa[j], g, fma(qb[j], rv, qc[j] * dprev)))));
      }
    } else {
      // A row off the cached factorisation: a locked row (identity, rhs psi)
      // or the reference's recurrence recomputed (thomas_solver.hpp:382-395),
      // with its derivative.
      double* p = V.rp(i);
      double c;
      bool singular = false;
      double tc[ND];
      if (lock) {
        dcur = psi_i;
        c = 0.0;
#pragma unroll
        for (int j = 0; j < ND; ++j) tdcur[j] = tc[j] = 0.0;
        fresh = true;
      } else {
        double rhs, trhs[ND];
        if (K == kStage1) {
          const double el = p[A_E1L0 * kTile], ed = p[A_E1D0 * kTile], eu = p[A_E1U0 * kTile];
          rhs = fma(el, um, fma(ed, u0, eu * rv));
#pragma unroll
          for (int j = 0; j < ND; ++j) {
            const double gl = W.at(j, T_JL, i), gd = W.at(j, T_JD, i), gu = W.at(j, T_JU, i);
            trhs[j] = fma(el, tum[j], fma(ed, tu0[j], fma(eu, qv[j],
                      wst * fma(gl, um, fma(gd, u0, gu * rv)))));
          }
        } else if (K == kStage2) {
          rhs = fma(alpha, g, beta * rv);
#pragma unroll
          for (int j = 0; j < ND; ++j) trhs[j] = fma(alpha, qn[j], beta * qv[j]);
        } else {
          rhs = g;
#pragma unroll
          for (int j = 0; j < ND; ++j) trhs[j] = qn[j];
        }
        const double l = p[aL * kTile];
        const double denom = fma(-l, cprev, p[aDg * kTile]);
        singular = fabs(denom) < 1e-15;
        const double inv = 1.0 / denom;
        const double up = p[aU * kTile];
        c = up * inv;
        dcur = fma(-l, dprev, rhs) * inv;
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          const double tl = -wst * W.at(j, T_JL, i);
          const double tdg = -wst * W.at(j, T_JD, i);
          const double tup = -wst * W.at(j, T_JU, i);
          const double tden = tdg - tl * cprev - l * tcprev[j];
          tc[j] = (tup - c * tden) * inv;
          tdcur[j] = (trhs[j] - tl * dprev - l * tdprev[j] - dcur * tden) * inv;
        }
        fresh = always_fresh || __double_as_longlong(-c) != __double_as_longlong(p[aNC * kTile]);
      }
      // rows between the previous off-cache row and this one keep their
      // cached factors in the scratch rows, so [lo, hi] stays contiguous
      if (hi >= 0 && i > hi + 1)
        for (int q = hi + 1; q < i; ++q) {
          V.at(A_CP, q) = V.at(aNC, q);
#pragma unroll
          for (int j = 0; j < ND; ++j) W.at(j, T_CP, q) = W.at(j, tNC, q);
        }
      p[A_CP * kTile] = -c;
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        W.at(j, T_CP, i) = -tc[j];
        tcprev[j] = tc[j];
      }
      lo = lo == INT_MAX ? i : lo;
      hi = i;
      cprev = c;
      if (singular) st = kStatusSolver;
    }
    V.at(A_D, i) = dcur;
    dprev = dcur;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      W.at(j, T_D, i) = tdcur[j];
      tdprev[j] = tdcur[j];
    }
    if (K == kStage1) {
      um = u0;
      u0 = rv;
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        tum[j] = tu0[j];
        tu0[j] = qv[j];
      }
    }
  };
  int i = 1;
  for (const int e1 = min(flo - 1, stop); i <= e1; ++i) row(i, std::false_type{});
  for (const int e2 = min(fhi, stop); i <= e2; ++i) row(i, std::true_type{});
  for (; i <= stop; ++i) row(i, std::false_type{});

  // ---- projected back substitution; the last row is the Dirichlet value
  if (!live) return st;
  __threadfence_block();
  const double psi_last = V.at(A_PSI, n - 1);
  double xnext = dmax_ref(bcr, psi_last);
  double txnext[ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) txnext[j] = bcr < psi_last ? 0.0 : tbcr.v[j];
  const int top = n - 2;
  for (int j = 0; j < RG::kAhead; ++j) {
    if (top - j >= 1) issue_bwd_t<K, ND>(V, W, R, top - j, lo, hi);
    cp_commit();
  }
  for (int i = top; i >= 1; --i) {
    cp_wait<RG::kAhead - 1>();
    const double* s = R + (i % RG::kSlots) * RG::kSlot;
    const double rnc = s[0], rpsi = s[kTile], rd = s[2 * kTile];
    double rtnc[ND], rtd[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      rtnc[j] = s[(3 + 2 * j) * kTile];
      rtd[j] = s[(4 + 2 * j) * kTile];
    }
    if (i - RG::kAhead >= 1) issue_bwd_t<K, ND>(V, W, R, i - RG::kAhead, lo, hi);
    cp_commit();
    const double nc = rnc;  // the ring holds the right -c' (and derivatives) for this row
    const double unc = fma(nc, xnext, rd);
    const bool act = binds(unc, rpsi);
    const double xv = act ? rpsi : unc;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      const double tnc = rtnc[j];
      const double tx = act ? 0.0 : fma(nc, txnext[j], fma(tnc, xnext, rtd[j]));
      W.at(j, t_out, i) = tx;
      txnext[j] = tx;
    }
    V.at(a_out, i) = xv;
    xnext = xv;
  }
  V.at(a_out, 0) = bcl;
  V.at(a_out, n - 1) = bcr;
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    W.at(j, t_out, 0) = 0.0;
    W.at(j, t_out, n - 1) = tbcr.v[j];
  }
  return st;
}

}  // namespace

template <int ND>
__device__ __forceinline__ void march_tan_body(
    const TileDev* __restrict__ tiles, int ntiles, const OptDev* __restrict__ opts,
    double* __restrict__ pool, double* __restrict__ tpool, const uint8_t* __restrict__ flags,
    const int32_t* __restrict__ mode, int32_t* __restrict__ status, int* __restrict__ queue,
    TanConst tc, MarchConst mc) {
  using RG = TanRing<ND>;
  const int lane = threadIdx.x & (kTile - 1);
  __shared__ double ring[2][RG::kWarp];  // one ring per warp (64 threads)
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(queue, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ntiles) break;
    const TileDev td = tiles[t];
    const int k = td.first + lane;
    const bool active = lane < td.count && (!mc.active || mc.active[k]) && k < mc.tv_first;
    if (!__any_sync(0xffffffffu, active)) continue;
    OptDev o{};
    int32_t md = 0;
    if (active) {
      o = opts[k];
      md = mode[k];
    }
    const bool nocache = (md & 1) != 0;
    const int n = active ? o.n : 0;
    const int nt = active ? o.nt : 0;
    const TileView V{pool + td.off + lane, td.nx};
    const TanView<ND> W{tpool + tan_off<ND>(td) + lane};
    const uint8_t* F = flags + td.foff + lane;
    double* R = ring[threadIdx.x / kTile];
    int flo = INT_MAX, fhi = -1, ncand = 0;
    for (int i = 1; i < n - 1; ++i)
      if (ROW(F, i)) {
        flo = min(flo, i);
        fhi = i;
        ++ncand;
      }
    const int cflo = flo, cfhi = fhi;
    const bool cexact = ncand == 0 || ncand == cfhi - cflo + 1;
    flo = __reduce_min_sync(0xffffffffu, flo);
    fhi = __reduce_max_sync(0xffffffffu, fhi);
    int32_t st = kStatusOk;
    const double dt = o.dt;
    const double w1 = mc.gamma * dt / 2.0;
    const double w2 = (1.0 - mc.gamma) * dt / (2.0 - mc.gamma);
    const double wr = 0.5 * dt;
    // Right boundary e^{x_{n-1}} - e^{-r t} of a call and its tangent along
    // the rate (t e^{-r t}); zero for puts and other directions.
    auto bc_r = [&](double tt, TanVec<ND>* tb) {
#pragma unroll
      for (int j = 0; j < ND; ++j) tb->v[j] = 0.0;
      if (o.is_put) return 0.0;
      const double e = exp(-o.r * tt);
#pragma unroll
      for (int j = 0; j < ND; ++j)
        if (tc.dirs[j] == kDirRate) tb->v[j] = tt * e;
      return o.exp_xr - e;
    };
    TanVec<ND> tb;
    int step = 0;
    if (mc.rannacher) {
      const double t_mid = 0.0 + 0.5 * dt;
      const double t_next = 0.0 + dt;
      double bcr = bc_r(t_mid, &tb);
      st = stage_t<kRannacher, ND>(active, n, V, W, F, nocache, o.bc_left, bcr, tb, mc.alpha,
                                   mc.beta, wr, A_U, A_G, T_U, T_G, st, flo, fhi, R, cflo, cfhi,
                                   cexact);
      bcr = bc_r(t_next, &tb);
      st = stage_t<kRannacher, ND>(active, n, V, W, F, nocache, o.bc_left, bcr, tb, mc.alpha,
                                   mc.beta, wr, A_G, A_U, T_G, T_U, st, flo, fhi, R, cflo, cfhi,
                                   cexact);
      step = 1;
    }
    for (; step < td.nt; ++step) {
      const bool live = active && step < nt && st == kStatusOk;
      const double tt = static_cast<double>(step) * dt;
      const double t1 = tt + mc.gamma * dt;
      const double tn = static_cast<double>(step + 1) * dt;
      const bool last = (step == nt - 1);
      double bcr = bc_r(t1, &tb);
      st = stage_t<kStage1, ND>(live, n, V, W, F, nocache, o.bc_left, bcr, tb, mc.alpha, mc.beta,
                                w1, A_U, A_G, T_U, T_G, st, flo, fhi, R, cflo, cfhi, cexact);
      bcr = bc_r(tn, &tb);
      st = stage_t<kStage2, ND>(live, n, V, W, F, nocache, o.bc_left, bcr, tb, mc.alpha, mc.beta,
                                w2, A_G, last ? A_G : A_U, T_G, last ? T_G : T_U, st, flo, fhi, R,
                                cflo, cfhi, cexact);
    }
    if (active) status[k] = st;
  }
}

// ---------------------------------------------------------- tangent outputs --
// Per option: value and delta (AmericanOptionResult::value_at / delta), then
// dV/dK and the derivative along each direction from the tangent's spline.
// out: kTanOutStride(ND) doubles per sorted option
// {value, delta, dV/dK, dV/d(direction 0), ...}; NaN for a failed option.
template <int ND>
__device__ __forceinline__ void outputs_tan_body(const TileDev* __restrict__ tiles, int ntiles,
                                   const OptDev* __restrict__ opts, const double* __restrict__ xs,
                                   double* __restrict__ pool, const double* __restrict__ tpool,
                                   const int32_t* __restrict__ mode,
                                   const int32_t* __restrict__ status, MarchConst mc,
                                   double* __restrict__ out) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int t = gt / kTile, lane = gt % kTile;
  if (t >= ntiles) return;
  const TileDev td = tiles[t];
  if (lane >= td.count) return;
  const int k = td.first + lane;
  if (mc.active && !mc.active[k]) return;
  constexpr int S = tan_out_stride(ND);
  double* res = out + static_cast<size_t>(S) * k;
  if (status[k] != kStatusOk || k >= mc.tv_first) {
    for (int j = 0; j < S; ++j) res[j] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const OptDev o = opts[k];
  const TileView V{pool + td.off + lane, td.nx};
  const TanView<ND> W{const_cast<double*>(tpool) + tan_off<ND>(td) + lane};
  const double* X = xs + td.xoff + lane;
  const bool swap = mc.rannacher && o.nt == 1;
  const int au = swap ? A_U : A_G;
  const int tu = swap ? T_U : T_G;
  const SplineScratch Sc{&V.at(A_CP, 0), &V.at(A_D, 0), kRowStride};
  const int n = o.n;
  const double xsp = o.x_spot;
  const int iv = find_interval(X, n, xsp);
  double sv, sd;
  spline_at(X, V, au, n, xsp, iv, Sc, &sv, &sd);
  const bool below = xsp <= ROW(X, 0), above = xsp >= ROW(X, n - 1);
  const int edge = below ? 0 : n - 1;
  double value, dK;
  bool clamp0 = false;
  if (below || above) {
    value = V.at(au, edge) * o.strike;
    dK = V.at(au, edge);
  } else {
    clamp0 = !(0.0 < sv);
    value = (clamp0 ? 0.0 : sv) * o.strike;
    dK = clamp0 ? 0.0 : sv - sd;
  }
  res[0] = value;
  res[1] = sd * (o.strike / o.spot);
  res[2] = dK;
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    double tv, tdv;
    spline_eval(X, [&](int i) { return W.at(j, tu, i); }, n, xsp, iv, Sc, &tv, &tdv);
    double dj;
    if (below || above) dj = W.at(j, tu, edge);
    else dj = clamp0 ? 0.0 : tv;
    res[3 + j] = dj * o.strike;
  }
}

// Concrete kernels, one per direction count (1: volatility, for Newton
// steps on the implied volatility; 3: volatility, rate, dividend yield).
#define MGPU_TAN_KERNELS(ND)                                                                   \
  __global__ void prep_tan_kernel_##ND(const TileDev* __restrict__ tiles, int ntiles,          \
                                       const OptDev* __restrict__ opts,                        \
                                       const double* __restrict__ xs,                          \
                                       const double* __restrict__ pool,                        \
                                       double* __restrict__ tpool, TanConst tc, MarchConst mc) { \
    prep_tan_body<ND>(tiles, ntiles, opts, xs, pool, tpool, tc, mc);                           \
  }                                                                                            \
  __global__ void __launch_bounds__(64) march_tan_kernel_##ND(                                 \
      const TileDev* __restrict__ tiles, int ntiles, const OptDev* __restrict__ opts,          \
      double* __restrict__ pool, double* __restrict__ tpool,                                   \
      const uint8_t* __restrict__ flags, const int32_t* __restrict__ mode,                     \
      int32_t* __restrict__ status, int* __restrict__ queue, TanConst tc, MarchConst mc) {     \
    march_tan_body<ND>(tiles, ntiles, opts, pool, tpool, flags, mode, status, queue, tc, mc);  \
  }                                                                                            \
  __global__ void outputs_tan_kernel_##ND(                                                     \
      const TileDev* __restrict__ tiles, int ntiles, const OptDev* __restrict__ opts,          \
      const double* __restrict__ xs, double* __restrict__ pool,                                \
      const double* __restrict__ tpool, const int32_t* __restrict__ mode,                      \
      const int32_t* __restrict__ status, MarchConst mc, double* __restrict__ out) {           \
    outputs_tan_body<ND>(tiles, ntiles, opts, xs, pool, tpool, mode, status, mc, out);         \
  }
MGPU_TAN_KERNELS(1)
MGPU_TAN_KERNELS(3)
#undef MGPU_TAN_KERNELS

// ------------------------------------------------------------------- host --

int64_t tan_pool_doubles(int nd, int64_t pool_doubles) {
  return pool_doubles / A_COUNT * nd * T_COUNT;
}

namespace {

template <int ND>
struct TanKernels;
template <>
struct TanKernels<1> {
  static constexpr auto prep = prep_tan_kernel_1;
  static constexpr auto march = march_tan_kernel_1;
  static constexpr auto outputs = outputs_tan_kernel_1;
};
template <>
struct TanKernels<3> {
  static constexpr auto prep = prep_tan_kernel_3;
  static constexpr auto march = march_tan_kernel_3;
  static constexpr auto outputs = outputs_tan_kernel_3;
};

template <int ND>
int tan_blocks_per_sm() {
  static int bps = 0;
  if (bps == 0) {
    int v = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, TanKernels<ND>::march, 64, 0),
          "occupancy");
    bps = std::max(1, v);
  }
  return bps;
}

template <int ND>
void tan_launch_nd(cudaStream_t st, int num_sms, const TileDev* tiles, int ntiles,
                   const OptDev* opts, const double* xs, double* pool, double* tpool,
                   uint8_t* flags, int32_t* mode, int32_t* status, int* queue, const TanConst& tc,
                   const MarchConst& mc, double* out) {
  const int threads = ntiles * kTile;
  prep_kernel<<<(threads + 127) / 128, 128, 0, st>>>(tiles, ntiles, opts, xs, pool, flags, mode,
                                                     mc);
  check(cudaGetLastError(), "tangent march: setup launch");
  TanKernels<ND>::prep<<<(threads + 127) / 128, 128, 0, st>>>(tiles, ntiles, opts, xs, pool,
                                                              tpool, tc, mc);
  check(cudaGetLastError(), "tangent march: tangent setup launch");
  const int blocks =
      std::max(1, std::min<int>(num_sms * tan_blocks_per_sm<ND>(), (ntiles + 1) / 2));
  TanKernels<ND>::march<<<blocks, 64, 0, st>>>(tiles, ntiles, opts, pool, tpool, flags, mode,
                                               status, queue, tc, mc);
  check(cudaGetLastError(), "tangent march: march launch");
  TanKernels<ND>::outputs<<<(threads + 127) / 128, 128, 0, st>>>(tiles, ntiles, opts, xs, pool,
                                                                 tpool, mode, status, mc, out);
  check(cudaGetLastError(), "tangent march: outputs launch");
}

}  // namespace

void tan_launch(int nd, void* stream, int num_sms, const TileDev* tiles, int ntiles,
                const OptDev* opts, const double* xs, double* pool, double* tpool,
                uint8_t* flags, int32_t* mode, int32_t* status, int* queue, const TanConst& tc,
                const MarchConst& mc, double* out) {
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (nd == 1)
    tan_launch_nd<1>(st, num_sms, tiles, ntiles, opts, xs, pool, tpool, flags, mode, status, queue,
                     tc, mc, out);
  else if (nd == 3)
    tan_launch_nd<3>(st, num_sms, tiles, ntiles, opts, xs, pool, tpool, flags, mode, status, queue,
                     tc, mc, out);
  else
    throw CudaError("tangent march: 1 or 3 directions");
}

namespace {

// The batch pipeline (validation, grids, sort, tiles, upload) and the
// tangent march along nd directions; results into MangoGpuGreeksOut slots.
MangoStatus tan_batch(MangoGpuContext* ctx, const MangoPricingParams* params, uint64_t n,
                      const MangoGpuGrid* grids, uint64_t grid_stride, int nd,
                      MangoGpuGreeksOut* out, uint64_t* out_failed, MangoError* err) {
  if (!ctx || (n > 0 && (!params || !out))) {
    set_err(err, MANGO_ERR_VALIDATION, "null context, params or out");
    return MANGO_ERR_VALIDATION;
  }
  if (n > (1ull << 30)) {
    set_err(err, MANGO_ERR_VALIDATION, "batch above 2^30 options");
    return MANGO_ERR_VALIDATION;
  }
  if (out_failed) *out_failed = 0;
  if (n == 0) return MANGO_OK;
  MangoGpuBatch* b = nullptr;
  DevBuf d_tpool, d_tout;
  // the split three-direction march: two more primal pools, three tangent
  // pools and outputs, per extra direction its flags, modes and statuses
  DevBuf d_split[2], d_split_t[3], d_split_o[3], d_split_aux[2][3];
  cudaEvent_t split_ev[2] = {nullptr, nullptr};
  struct Release {
    MangoGpuBatch** b;
    std::vector<DevBuf*> bufs;
    cudaEvent_t* ev;
    ~Release() {
      if (*b) destroy_batch(*b);
      for (DevBuf* x : bufs) x->release();
      for (int j = 0; j < 2; ++j)
        if (ev[j]) cudaEventDestroy(ev[j]);
    }
  } release{&b,
            {&d_tpool, &d_tout, &d_split[0], &d_split[1], &d_split_t[0], &d_split_t[1],
             &d_split_t[2], &d_split_o[0], &d_split_o[1], &d_split_o[2], &d_split_aux[0][0],
             &d_split_aux[0][1], &d_split_aux[0][2], &d_split_aux[1][0], &d_split_aux[1][1],
             &d_split_aux[1][2]},
            split_ev};
  try {
    check(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int64_t nn = static_cast<int64_t>(n);
    std::vector<Resolved> res(static_cast<size_t>(nn));
    std::vector<std::string> msg(static_cast<size_t>(nn));
    parallel_for(nn, [&](int64_t i) {
      thread_local std::vector<double> scratch;
      Resolved& r = res[i];
      r.orig = static_cast<int32_t>(i);
      // constant rates and continuous dividends only (the cached march)
      std::string m = validate(params[i], false);
      if (m.empty()) {
        MangoGpuGrid g{};
        g.kind = MANGO_GPU_GRID_AUTO;
        if (grids) g = grids[grid_stride ? i : 0];
        m = resolve(params[i], g, &r, &scratch);
      }
      if (!m.empty()) {
        r.status = MANGO_ERR_VALIDATION;
        msg[i] = m;
      }
    });
    b = create_batch_resolved(ctx, params, std::move(res), std::move(msg), nullptr);
    for (auto& e : split_ev) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    const int64_t m = static_cast<int64_t>(b->order.size());
    const int S = tan_out_stride(nd);
    std::vector<double> hout(static_cast<size_t>(m) * S);
    std::vector<int32_t> hst(static_cast<size_t>(m));
    cudaStream_t st = b->stream;
    if (m > 0) {
      const int64_t pool_doubles =
          static_cast<int64_t>(b->d_pool.cap / sizeof(double));
      double* tpool = static_cast<double*>(
          d_tpool.get(sizeof(double) * static_cast<size_t>(tan_pool_doubles(nd, pool_doubles))));
      double* dout = static_cast<double*>(d_tout.get(sizeof(double) * hout.size()));
      TanConst tc{};
      tc.dirs[0] = kDirSigma;
      tc.dirs[1] = kDirRate;
      tc.dirs[2] = kDirDividend;
      check(cudaMemsetAsync(b->d_queue.p, 0, sizeof(int) * 4, st), "memset queue");
      check(cudaEventRecord(b->ev[2], st), "event");
      // A batch whose three single-direction marches still fit one wave of
      // resident warps runs them side by side on three streams, each with its
      // own primal pool: the FP64 work grows by a third (the primal is
      // marched three times), but three times as many warps share the SM
      // sub-partitions of a launch that one warp per tile leaves
      // latency-bound (16,384 options: 512 tiles for 608 sub-partitions).
      const int wave1 = ctx->num_sms * tan_blocks_per_sm<1>() * 2;
      if (nd == 3 && 3 * b->ntiles <= wave1) {
        check(cudaEventRecord(b->ev[3], st), "event");
        cudaStream_t sd[3] = {st, ctx->aux[0], ctx->aux[1]};
        const size_t pool_bytes = sizeof(double) * static_cast<size_t>(pool_doubles);
        double* pools[3] = {b->d_pool.as<double>(), static_cast<double*>(d_split[0].get(pool_bytes)),
                            static_cast<double*>(d_split[1].get(pool_bytes))};
        const size_t t1 = sizeof(double) * static_cast<size_t>(tan_pool_doubles(1, pool_doubles));
        const size_t nflags = b->d_flags.cap;
        const size_t o1 = sizeof(double) * static_cast<size_t>(m) * tan_out_stride(1);
        for (int d = 0; d < 3; ++d) {
          if (d > 0) check(cudaStreamWaitEvent(sd[d], b->ev[3], 0), "stream wait");
          TanConst td{};
          td.dirs[0] = tc.dirs[d];
          uint8_t* fl = d == 0 ? b->d_flags.as<uint8_t>()
                               : static_cast<uint8_t*>(d_split_aux[d - 1][0].get(nflags));
          int32_t* md = d == 0 ? b->d_mode.as<int32_t>()
                               : static_cast<int32_t*>(d_split_aux[d - 1][1].get(sizeof(int32_t) * m));
          int32_t* sts = d == 0 ? b->d_status.as<int32_t>()
                                : static_cast<int32_t*>(d_split_aux[d - 1][2].get(sizeof(int32_t) * m));
          tan_launch(1, sd[d], ctx->num_sms, b->d_tiles.as<TileDev>(), b->ntiles,
                     b->d_opts.as<OptDev>(), b->d_xs.as<double>(), pools[d],
                     static_cast<double*>(d_split_t[d].get(t1)), fl, md, sts,
                     b->d_queue.as<int>() + d, td, b->mc,
                     static_cast<double*>(d_split_o[d].get(o1)));
          if (d > 0) {
            check(cudaEventRecord(split_ev[d - 1], sd[d]), "event");
            check(cudaStreamWaitEvent(st, split_ev[d - 1], 0), "stream wait");
          }
        }
        check(cudaEventRecord(b->ev[4], st), "event");
        std::vector<double> h1(static_cast<size_t>(m) * tan_out_stride(1));
        std::vector<int32_t> hs(static_cast<size_t>(m));
        for (int d = 0; d < 3; ++d) {
          check(cudaMemcpyAsync(h1.data(), d_split_o[d].p, o1, cudaMemcpyDeviceToHost, st),
                "D2H tangent results");
          const void* src = d == 0 ? b->d_status.p : d_split_aux[d - 1][2].p;
          check(cudaMemcpyAsync(hs.data(), src, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, st),
                "D2H status");
          check(cudaStreamSynchronize(st), "stream synchronize");
          for (int64_t k = 0; k < m; ++k) {
            const double* h = h1.data() + static_cast<size_t>(k) * tan_out_stride(1);
            double* o = hout.data() + static_cast<size_t>(k) * S;
            if (d == 0) {
              o[0] = h[0];  // value, delta, dV/dK from the volatility march
              o[1] = h[1];
              o[2] = h[2];
              hst[k] = hs[k];
            } else if (hst[k] == kStatusOk) {
              hst[k] = hs[k];
            }
            o[3 + d] = h[3];
          }
        }
      } else {
        tan_launch(nd, st, ctx->num_sms, b->d_tiles.as<TileDev>(), b->ntiles,
                   b->d_opts.as<OptDev>(), b->d_xs.as<double>(), b->d_pool.as<double>(), tpool,
                   b->d_flags.as<uint8_t>(), b->d_mode.as<int32_t>(), b->d_status.as<int32_t>(),
                   b->d_queue.as<int>(), tc, b->mc, dout);
        check(cudaEventRecord(b->ev[4], st), "event");
        check(cudaMemcpyAsync(hout.data(), dout, sizeof(double) * hout.size(),
                              cudaMemcpyDeviceToHost, st),
              "D2H tangent results");
        check(cudaMemcpyAsync(hst.data(), b->d_status.p, sizeof(int32_t) * m,
                              cudaMemcpyDeviceToHost, st),
              "D2H status");
        check(cudaStreamSynchronize(st), "stream synchronize");
      }
    }
    const double nan = std::nan("");
    uint64_t failed = 0;
    std::string first;
    for (int64_t i = 0; i < nn; ++i) {
      MangoGpuGreeksOut& g = out[i];
      g = MangoGpuGreeksOut{};
      g.base.status = b->res[i].status;
      g.base.n_space = static_cast<int32_t>(b->res[i].spec.n);
      g.base.n_time = static_cast<int32_t>(b->res[i].nt);
      g.base.value = g.base.delta = g.base.gamma = g.base.theta = nan;
      g.vega = g.rho = g.dividend_rho = g.dstrike = nan;
    }
    for (int64_t s = 0; s < m; ++s) {
      MangoGpuGreeksOut& g = out[b->order[s]];
      const double* h = hout.data() + static_cast<size_t>(s) * S;
      g.base.status = hst[s];
      if (hst[s] != MANGO_OK) continue;
      g.base.value = h[0];
      g.base.delta = h[1];
      g.dstrike = h[2];
      g.vega = h[3];
      if (nd == 3) {
        g.rho = h[4];
        g.dividend_rho = h[5];
      }
    }
    for (int64_t i = 0; i < nn; ++i)
      if (out[i].base.status != MANGO_OK && failed++ == 0)
        first = b->msgs[i].empty() ? "solver failure" : b->msgs[i];
    Stats& S2 = ctx->stats;
    S2 = Stats{};
    float ms = 0.f;
    if (m > 0 && cudaEventElapsedTime(&ms, b->ev[2], b->ev[4]) == cudaSuccess) S2.march_ms = ms;
    cudaGetLastError();
    S2.options = nn;
    S2.tiles = b->ntiles;
    S2.host_prep_ms = b->host_prep_ms;
    S2.kernel_launches = m > 0 ? (nd == 3 && 3 * b->ntiles <= ctx->num_sms * tan_blocks_per_sm<1>() * 2 ? 12 : 4) : 0;
    if (out_failed) *out_failed = failed;
    if (failed == n) {
      set_err(err, MANGO_ERR_VALIDATION, "every option failed: " + first);
      return MANGO_ERR_VALIDATION;
    }
    if (failed && err) set_err(err, MANGO_OK, first);
    return MANGO_OK;
  } catch (const std::exception& e) {
    set_err(err, MANGO_ERR_SOLVER, e.what());
    return MANGO_ERR_SOLVER;
  }
}

}  // namespace
}  // namespace mgpu

extern "C" MangoStatus mango_gpu_price_american_tangent_batch(
    MangoGpuContext* ctx, const MangoPricingParams* params, uint64_t n, const MangoGpuGrid* grids,
    uint64_t grid_stride, MangoGpuGreeksOut* out, uint64_t* out_failed, MangoError* err) {
  return mgpu::tan_batch(ctx, params, n, grids, grid_stride, 3, out, out_failed, err);
}

extern "C" MangoStatus mango_gpu_price_american_vega_batch(
    MangoGpuContext* ctx, const MangoPricingParams* params, uint64_t n, const MangoGpuGrid* grids,
    uint64_t grid_stride, MangoGpuGreeksOut* out, uint64_t* out_failed, MangoError* err) {
  return mgpu::tan_batch(ctx, params, n, grids, grid_stride, 1, out, out_failed, err);
}
