// wmarch.cu -- the American march with one warp per option (warp-cooperative
// projected Thomas), for launches whose options are too few to fill the GPU
// with one lane each: the last evaluations of a batched IV, the price-table
// sweep (200 slices), and small batches.
//
// The arithmetic is march.cu's (the reference's PDESolver::solve with the
// Rannacher start, TR-BDF2 stages, the projected stage with the deep-ITM lock
// and solve_thomas_projected, src/pde/internal/pde_solver.hpp:114-178,
// 342-447, 525-729, src/math/thomas_solver.hpp:321-420) on the same cached,
// time-invariant factorisation that prep_kernel builds; only the order of
// the two serial recurrences changes:
//  * grid row i belongs to lane i / R (R = ceil(n / 32) rows per lane); all
//    of an option's rows live in the warp's shared memory for the whole
//    march, so no time step touches HBM;
//  * forward elimination d'_i = a_i + m_i d'_{i-1} is an affine recurrence:
//    each lane composes its R row maps, a 5-level shuffle scan composes the
//    lanes, and each lane then re-runs its rows from its exact input with the
//    serial kernel's expression (fma(m, d'_{i-1}, a));
//  * the projected back substitution x_i = max(d'_i + nc_i x_{i+1}, psi_i) is
//    a chain of maps x -> clamp(beta x + alpha, lo, hi), a family closed
//    under composition, so it scans the same way (downwards), and each lane
//    re-runs its rows with the serial expression;
//  * the deep-ITM lock (pde_solver.hpp:635-680) is tested per row in
//    parallel; where a row locks, one lane recomputes the factorisation of
//    the following rows exactly as the reference does (thomas_solver.hpp:
//    382-395) until it agrees with the cached one again (3-4 rows), and the
//    scans take those rows' factors.  The Rannacher half steps have no cached
//    factorisation and are factored the same way, serially.
// Only the association at the 32 lane boundaries differs from the
// thread-per-option march, so results agree to rounding.
//
// Cost: about 8 FP64 instructions per row and stage for the map compositions
// plus 5 shuffle-scan levels, several times the FP64 work of the
// thread-per-option march per option, but the march of one option takes
// ~500 short scan rounds instead of 500 x n dependent row updates: it wins
// when there are fewer options than resident warps can hold in lanes.
#include "march_dev.cuh"

#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include <cstdlib>

#include "engine.hpp"
#include "wmarch.cuh"

namespace mgpu {
namespace {

// Shared-memory arrays per warp, layout [array][r][lane] (row i of the
// option at r = i % R, lane = i / R): conflict-free for a fixed r.
enum WArray : int {
  W_PSI = 0,
  W_E1L, W_E1D, W_E1U, W_N1H, W_NC1,  // stage 1 cached row factors
  W_A2H, W_B2H, W_N2H, W_NC2,         // stage 2 cached row factors
  W_L1, W_D1, W_U1, W_L2, W_D2, W_U2, // stage matrix bands (rows off the cache)
  W_U, W_G, W_D,                      // state u^n, u^{n+gamma}, Thomas d'
  W_MC, W_MI,                         // -c' and 1 / pivot of rows off the cache (stage 1)
  W_MC2, W_MI2,                       //   the same for stage 2
  W_FL,                               // lock-candidate flag (0 / 1)
  kWArrays
};
// Row modes of a stage, per row (bytes after the double arrays).
constexpr unsigned char kRowCached = 0, kRowLocked = 1, kRowOff = 2;
constexpr double kBig = 1e300;  // "no bound" of a clamp map
// Options of a large uneven batch that may go to the warp march beside the
// thread march (two warp blocks per SM, a few options each).  With the
// thread march's tiles assigned to SM sub-partitions, caps of 0, 304, 456,
// 608, 760, 912, 1216 and 2432 options measured 398, 360, 357, 355, 361,
// 382, 407 and 527 ms per launch on the 65,536-option uneven batch.
constexpr int64_t kLongWarpOptions = 608;

// R rows per lane, a compile-time constant: every row loop unrolls and
// every shared-memory address is a constant offset from the lane's column.
template <int R>
struct WView {
  double* s;
  unsigned char* md;  // row modes [r][lane]
  __device__ __forceinline__ double& atl(int a, int r, int lane) const {
    return s[(a * R + r) * 32 + lane];
  }
};

// The factor run of one stage kind that restarted after row L, kept in the
// stage's -c' / inverse-pivot arrays for rows (L, H] (lane 0's walk): a walk
// that restarts after the same row takes them instead of dividing again.
struct RunMemo {
  int L = -2, H = -2;
  int done = 0;  // the run ended in (L, H]: it re-converged at H or reached row n - 2
};

// x -> min(max(b x + a, lo), hi)
struct Clamp {
  double b, a, lo, hi;
};

// outer o applied after inner f
__device__ __forceinline__ Clamp compose(const Clamp& o, const Clamp& f) {
  Clamp h;
  h.b = o.b * f.b;
  h.a = fma(o.b, f.a, o.a);
  const double t1 = fma(o.b, f.lo, o.a), t2 = fma(o.b, f.hi, o.a);
  const bool pos = !(o.b < 0.0);
  const double lo1 = pos ? t1 : t2, hi1 = pos ? t2 : t1;
  h.lo = fmin(fmax(lo1, o.lo), o.hi);
  h.hi = fmin(fmax(hi1, o.lo), o.hi);
  return h;
}

__device__ __forceinline__ double apply(const Clamp& c, double x) {
  return fmin(fmax(fma(c.b, x, c.a), c.lo), c.hi);
}

// x -> max(b x + a, lo) with b >= 0: the back-substitution maps whenever
// every -c' of the stage is non-negative (the usual case: the implicit
// matrix is an M-matrix, so its upper factor has non-positive c').  Closed
// under composition without an upper bound, at half the arithmetic.
struct Mono {
  double b, a, lo;
};
__device__ __forceinline__ Mono compose(const Mono& o, const Mono& f) {
  return Mono{o.b * f.b, fma(o.b, f.a, o.a), fmax(fma(o.b, f.lo, o.a), o.lo)};
}
__device__ __forceinline__ double apply(const Mono& c, double x) {
  return fmax(fma(c.b, x, c.a), c.lo);
}

__device__ __forceinline__ double shfl_up_d(double v, int d) {
  return __shfl_up_sync(0xffffffffu, v, d);
}
__device__ __forceinline__ double shfl_down_d(double v, int d) {
  return __shfl_down_sync(0xffffffffu, v, d);
}

enum StageKind { kRannacher = 0, kStage1 = 1, kStage2 = 2 };

// One projected implicit stage of one option on one warp:
//   kRannacher: rhs = guess = u_prev (array a_in), bands LR/DR/UR from the pool;
//   kStage1:    rhs = u + w1 L(u) of u^n (W_U), guess u^n, writes W_G;
//   kStage2:    rhs = alpha g + beta u^n (g = W_G), guess g, writes a_out.
// P: the option's rows in the tile pool (Rannacher bands); returns the status.
template <int K, int R>
__device__ int32_t wstage(RunMemo& memo, const WView<R>& W, const TileView& P, int n, bool nocache, int flo,
                          int fhi, double bcl, double bcr, double alpha, double beta, int a_in,
                          int a_out, int32_t st) {
  const int lane = threadIdx.x & 31;
  const bool always_fresh = (K == kRannacher) || nocache;
  const int a_guess = (K == kStage1) ? W_U : a_in;
  // ---- lock test per row (pde_solver.hpp:635-680), rows [flo, fhi]
  int last_lock = -1, first_lock = INT_MAX, nlock = 0;
  for (int r = 0; r < R; ++r) {
    const int i = lane * R + r;
    bool lock = false;
    if (i >= flo && i <= fhi && i >= 1 && i <= n - 2 && W.atl(W_FL, r, lane) != 0.0)
      lock = W.atl(a_guess, r, lane) - W.atl(W_PSI, r, lane) < 1e-8;
    W.md[r * 32 + lane] = lock ? kRowLocked : kRowCached;
    if (lock) {
      last_lock = i;
      first_lock = min(first_lock, i);
      ++nlock;
    }
  }
  last_lock = __reduce_max_sync(0xffffffffu, last_lock);
  first_lock = __reduce_min_sync(0xffffffffu, first_lock);
  nlock = __reduce_add_sync(0xffffffffu, nlock);
  const bool one_block = last_lock >= 0 && nlock == last_lock - first_lock + 1;
  // lane 0 keeps the memo; every lane reads it
  memo.L = __shfl_sync(0xffffffffu, memo.L, 0);
  memo.H = __shfl_sync(0xffffffffu, memo.H, 0);
  memo.done = __shfl_sync(0xffffffffu, memo.done, 0);
  __syncwarp();
  // One lock block ending where the memo's complete run restarted: the rows
  // off the cache are exactly the memo's, so every lane marks its own and
  // nothing is walked.
  const bool memo_run = K != kRannacher && !always_fresh && one_block && memo.done &&
                        memo.L == last_lock;
  if (memo_run) {
    for (int r = 0; r < R; ++r) {
      const int i = lane * R + r;
      if (i > memo.L && i <= memo.H) W.md[r * 32 + lane] = kRowOff;
    }
    __syncwarp();
  }
  // ---- rows off the cache: one lane walks them in order, as the serial
  // sweep does, from the first locked row (every row for the Rannacher
  // stages and an option without a usable cache) until the recomputed c'
  // is bit-identical to the cached one after the last locked row.
  if (!memo_run && (always_fresh || last_lock >= 0)) {
    if (lane == 0) {
      constexpr int aMC = (K == kStage2) ? W_MC2 : W_MC, aMI = (K == kStage2) ? W_MI2 : W_MI;
      constexpr bool kMemo = (K != kRannacher);
      // one lock block: its rows before the last need no visit
      int i = always_fresh ? 1 : (one_block ? last_lock : first_lock);
      double cprev = 0.0;  // c'_{i-1}: zero after a locked or Dirichlet row
      bool fresh = always_fresh;
      int run_l = always_fresh ? 0 : -1;  // the row the current run restarted after
      int last_off = -1;                  // the last row put off the cache
      int ri = i % R, li = i / R;  // row i at [ri][li], advanced without division
      for (; i <= n - 2; ++i, ri = (ri + 1 == R) ? 0 : ri + 1, li += (ri == 0) ? 1 : 0) {
        unsigned char& m = W.md[ri * 32 + li];
        if (m == kRowLocked) {
          cprev = 0.0;
          fresh = true;
          run_l = i;
          continue;
        }
        if (!fresh) {
          if (i > last_lock) break;
          continue;
        }
        double l, dg, up, nc_cached;
        if (K == kRannacher) {
          l = P.at(A_LR, i);
          dg = P.at(A_DR, i);
          up = P.at(A_UR, i);
          nc_cached = 0.0;
        } else if (K == kStage1) {
          l = W.atl(W_L1, ri, li);
          dg = W.atl(W_D1, ri, li);
          up = W.atl(W_U1, ri, li);
          nc_cached = W.atl(W_NC1, ri, li);
        } else {
          l = W.atl(W_L2, ri, li);
          dg = W.atl(W_D2, ri, li);
          up = W.atl(W_U2, ri, li);
          nc_cached = W.atl(W_NC2, ri, li);
        }
        double c;
        if (kMemo && run_l == memo.L && i <= memo.H) {
          c = -W.atl(aMC, ri, li);  // stored by the memo's run, with its inverse pivot
        } else {
          const double denom = fma(-l, cprev, dg);
          if (fabs(denom) < 1e-15) st = kStatusSolver;
          const double inv = 1.0 / denom;
          c = up * inv;
          W.atl(aMC, ri, li) = -c;
          W.atl(aMI, ri, li) = inv;
          if (kMemo) {
            if (run_l == memo.L && i == memo.H + 1) {
              memo.H = i;
            } else if (i == run_l + 1) {
              memo.L = run_l;
              memo.H = i;
            } else if (i > memo.L && i <= memo.H) {
              memo.H = i - 1;
            }
          }
        }
        m = kRowOff;
        fresh = always_fresh || __double_as_longlong(-c) != __double_as_longlong(nc_cached);
        cprev = c;
        last_off = i;
      }
      // the memo's run is complete when it is the last run and holds its
      // last row (re-convergence, or row n - 2)
      if (kMemo) memo.done = (run_l == memo.L && memo.H == last_off) ? 1 : 0;
    }
    st = __shfl_sync(0xffffffffu, st, 0);
    __syncwarp();
  }
  // ---- forward elimination: row maps d' = a + m d'_prev, composed per lane
  // then scanned across lanes (row 0: d'_0 = bcl, a constant map).
  auto row_map = [&](int r, double& a, double& m) {
    const int i = lane * R + r;
    if (i == 0) {
      a = bcl;
      m = 0.0;
      return;
    }
    if (i > n - 2) {  // the Dirichlet row n-1 and padding: identity
      a = 0.0;
      m = 1.0;
      return;
    }
    const unsigned char md = W.md[r * 32 + lane];
    if (md == kRowLocked) {
      a = W.atl(W_PSI, r, lane);
      m = 0.0;
      return;
    }
    double um = 0.0, u0 = 0.0, up = 0.0, g = 0.0, v = 0.0;
    if (K == kStage1) {
      // neighbours: the lane's own adjacent rows, or the next lane's edge
      um = r > 0 ? W.atl(W_U, r - 1, lane) : W.atl(W_U, R - 1, lane - 1);
      u0 = W.atl(W_U, r, lane);
      up = r + 1 < R ? W.atl(W_U, r + 1, lane) : W.atl(W_U, 0, lane + 1);
    } else if (K == kStage2) {
      g = W.atl(W_G, r, lane);
      v = W.atl(W_U, r, lane);
    } else {
      g = W.atl(a_in, r, lane);
    }
    if (md == kRowCached) {
      if (K == kStage1) {
        a = fma(W.atl(W_E1L, r, lane), um,
                fma(W.atl(W_E1D, r, lane), u0, W.atl(W_E1U, r, lane) * up));
        m = W.atl(W_N1H, r, lane);
      } else {  // kStage2 (the Rannacher stages never use the cache)
        a = fma(W.atl(W_A2H, r, lane), g, W.atl(W_B2H, r, lane) * v);
        m = W.atl(W_N2H, r, lane);
      }
      return;
    }
    // a row off the cache: d' = (rhs - l d'_prev) / pivot
    double rhs, l;
    if (K == kStage1) {
      // the stage-1 explicit stencil in its matrix form: (2 I - A1) u
      const double l1 = W.atl(W_L1, r, lane), d1 = W.atl(W_D1, r, lane),
                   u1 = W.atl(W_U1, r, lane);
      rhs = fma(-l1, um, fma(2.0 - d1, u0, -u1 * up));
      l = l1;
    } else if (K == kStage2) {
      rhs = fma(alpha, g, beta * v);
      l = W.atl(W_L2, r, lane);
    } else {
      rhs = g;
      l = P.at(A_LR, i);
    }
    const double inv = W.atl(K == kStage2 ? W_MI2 : W_MI, r, lane);
    a = rhs * inv;
    m = -l * inv;
  };
  // the multiplier of a row map again, without its constant term
  auto row_m = [&](int r) {
    const int i = lane * R + r;
    if (i == 0) return 0.0;
    if (i > n - 2) return 1.0;
    const unsigned char md = W.md[r * 32 + lane];
    if (md == kRowLocked) return 0.0;
    if (md == kRowCached) return W.atl(K == kStage1 ? W_N1H : W_N2H, r, lane);
    const double l = K == kStage1 ? W.atl(W_L1, r, lane)
                                  : (K == kStage2 ? W.atl(W_L2, r, lane) : P.at(A_LR, i));
    return -l * W.atl(K == kStage2 ? W_MI2 : W_MI, r, lane);
  };
  double A = 0.0, M = 1.0;
  for (int r = 0; r < R; ++r) {
    double a, m;
    row_map(r, a, m);
    W.atl(W_D, r, lane) = a;  // the constant term, reused below
    A = fma(m, A, a);
    M = m * M;
  }
  for (int off = 1; off < 32; off <<= 1) {
    const double oa = shfl_up_d(A, off), om = shfl_up_d(M, off);
    if (lane >= off) {
      A = fma(M, oa, A);
      M = M * om;
    }
  }
  double dprev = shfl_up_d(A, 1);  // d' at the top row of the lane below
  for (int r = 0; r < R; ++r) {
    const double d = fma(row_m(r), dprev, W.atl(W_D, r, lane));
    W.atl(W_D, r, lane) = d;
    dprev = d;
  }
  __syncwarp();
  // ---- projected back substitution: x_i = max(d'_i + nc_i x_{i+1}, psi_i),
  // the last row x_{n-1} = max(bcr, psi_{n-1}) (a constant map).
  auto row_nc = [&](int r) {
    const unsigned char md = W.md[r * 32 + lane];
    return md == kRowCached ? W.atl(K == kStage2 ? W_NC2 : W_NC1, r, lane)
                            : (md == kRowOff ? W.atl(K == kStage2 ? W_MC2 : W_MC, r, lane) : 0.0);
  };
  auto back_map = [&](int r) {
    const int i = lane * R + r;
    if (i >= n || i == 0) return Clamp{1.0, 0.0, -kBig, kBig};
    if (i == n - 1) return Clamp{0.0, bcr, W.atl(W_PSI, r, lane), kBig};
    return Clamp{row_nc(r), W.atl(W_D, r, lane), W.atl(W_PSI, r, lane), kBig};
  };
  // every suffix that reaches row n-1 holds its constant map: its value is x
  // at the lane's lowest row, and the lane above supplies the input of this
  // lane's top row
  bool nonneg = true;
  for (int r = 0; r < R; ++r) {
    const int i = lane * R + r;
    if (i >= 1 && i <= n - 2) nonneg = nonneg && !(row_nc(r) < 0.0);
  }
  double xnext;
  if (__all_sync(0xffffffffu, nonneg)) {
    Mono C{1.0, 0.0, -kBig};
    for (int r = R - 1; r >= 0; --r) {
      const Clamp m = back_map(r);
      C = compose(Mono{m.b, m.a, m.lo}, C);
    }
    for (int off = 1; off < 32; off <<= 1) {
      Mono o;
      o.b = shfl_down_d(C.b, off);
      o.a = shfl_down_d(C.a, off);
      o.lo = shfl_down_d(C.lo, off);
      if (lane + off < 32) C = compose(C, o);
    }
    xnext = shfl_down_d(apply(C, 0.0), 1);
  } else {
    Clamp C{1.0, 0.0, -kBig, kBig};
    for (int r = R - 1; r >= 0; --r) C = compose(back_map(r), C);
    for (int off = 1; off < 32; off <<= 1) {
      Clamp o;
      o.b = shfl_down_d(C.b, off);
      o.a = shfl_down_d(C.a, off);
      o.lo = shfl_down_d(C.lo, off);
      o.hi = shfl_down_d(C.hi, off);
      if (lane + off < 32) C = compose(C, o);
    }
    xnext = shfl_down_d(apply(C, 0.0), 1);
  }
  for (int r = R - 1; r >= 0; --r) {
    const int i = lane * R + r;
    if (i >= n) continue;
    double x;
    if (i == n - 1) {
      xnext = dmax_ref(bcr, W.atl(W_PSI, r, lane));
      x = bcr;  // apply_boundary_conditions after the solve (pde_solver.hpp:724-726)
    } else if (i == 0) {
      x = bcl;
    } else {
      x = proj_max(fma(row_nc(r), xnext, W.atl(W_D, r, lane)), W.atl(W_PSI, r, lane));
      xnext = x;
    }
    W.atl(a_out, r, lane) = x;
  }
  __syncwarp();
  return st;
}

__device__ __forceinline__ double right_bc(const OptDev& o, double t) {
  return o.is_put ? 0.0 : o.exp_xr - exp(-o.r * t);  // american_option.cpp:276-290
}

}  // namespace

// Persistent: each warp takes options (warp tiles wt[0..nwt) x 32 lanes) from
// the queue; R = rows per lane, at least that of the launch's widest option.
template <int R>
__device__ __forceinline__ void wmarch_body(
    double* wsm, const TileDev* __restrict__ tiles, const int32_t* __restrict__ wt, int nwt,
    const OptDev* __restrict__ opts, double* __restrict__ pool, const uint8_t* __restrict__ flags,
    const int32_t* __restrict__ mode, int32_t* __restrict__ status, int* __restrict__ queue,
    const MarchConst& mc) {
  const int lane = threadIdx.x & 31;
  const WView<R> W{wsm, reinterpret_cast<unsigned char*>(wsm + static_cast<size_t>(kWArrays) * R * 32)};
  for (;;) {
    int item = 0;
    if (lane == 0) item = atomicAdd(queue, 1);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= nwt * kTile) break;
    const int t = wt[item / kTile], l = item % kTile;
    const TileDev td = tiles[t];
    const int k = td.first + l;
    if (l >= td.count || (mc.active && !mc.active[k]) || k >= mc.tv_first) continue;
    const OptDev o = opts[k];
    const int n = o.n;
    if (n > 32 * R) {  // not sized for this launch (the host keeps it off)
      if (lane == 0) status[k] = kStatusSolver;
      continue;
    }
    const bool nocache = (mode[k] & 1) != 0;
    const TileView P{pool + td.off + l, td.nx};
    const uint8_t* F = flags + td.foff + l;
    // the option's rows into shared memory
    for (int r = 0; r < R; ++r) {
      const int i = lane * R + r;
      if (i >= n) continue;
      const double* p = P.rp(i);
      W.atl(W_PSI, r, lane) = p[A_PSI * kTile];
      W.atl(W_U, r, lane) = p[A_U * kTile];
      W.atl(W_FL, r, lane) = ROW(F, i) ? 1.0 : 0.0;
      if (i >= 1 && i <= n - 2) {
        W.atl(W_E1L, r, lane) = p[A_E1L * kTile];
        W.atl(W_E1D, r, lane) = p[A_E1D * kTile];
        W.atl(W_E1U, r, lane) = p[A_E1U * kTile];
        W.atl(W_N1H, r, lane) = p[A_N1H * kTile];
        W.atl(W_NC1, r, lane) = p[A_NC1 * kTile];
        W.atl(W_A2H, r, lane) = p[A_A2H * kTile];
        W.atl(W_B2H, r, lane) = p[A_B2H * kTile];
        W.atl(W_N2H, r, lane) = p[A_N2H * kTile];
        W.atl(W_NC2, r, lane) = p[A_NC2 * kTile];
        W.atl(W_L1, r, lane) = p[A_L1 * kTile];
        W.atl(W_D1, r, lane) = p[A_D1 * kTile];
        W.atl(W_U1, r, lane) = p[A_U1 * kTile];
        W.atl(W_L2, r, lane) = p[A_L2 * kTile];
        W.atl(W_D2, r, lane) = p[A_D2 * kTile];
        W.atl(W_U2, r, lane) = p[A_U2 * kTile];
      }
    }
    // lock-candidate rows: the block of flagged rows
    int flo = INT_MAX, fhi = -1;
    for (int r = 0; r < R; ++r) {
      const int i = lane * R + r;
      if (i >= 1 && i <= n - 2 && W.atl(W_FL, r, lane) != 0.0) {
        flo = min(flo, i);
        fhi = max(fhi, i);
      }
    }
    flo = __reduce_min_sync(0xffffffffu, flo);
    fhi = __reduce_max_sync(0xffffffffu, fhi);
    __syncwarp();
    int32_t st = kStatusOk;
    const double dt = o.dt;
    RunMemo memo1, memo2, memo_r;  // stage 1, stage 2; the Rannacher stages keep none
    int sp = 0, sc = 0;
    const int32_t* sidx = nullptr;
    double* sout = nullptr;
    if (mc.snap_idx) {
      sidx = mc.snap_idx + mc.snap_begin[k];
      sc = mc.snap_count[k];
      sout = mc.snap_out + mc.snap_off[k];
    }
    auto record = [&](int state, int arr) {
      while (sp < sc && sidx[sp] == state) {
        for (int r = 0; r < R; ++r) {
          const int i = lane * R + r;
          if (i < n) sout[static_cast<size_t>(sp) * n + i] = W.atl(arr, r, lane);
        }
        ++sp;
      }
    };
    record(0, W_U);
    int step = 0;
    if (mc.rannacher) {
      const double t_mid = 0.0 + 0.5 * dt;
      const double t_next = 0.0 + dt;
      st = wstage<kRannacher, R>(memo_r, W, P, n, nocache, flo, fhi, o.bc_left, right_bc(o, t_mid), mc.alpha,
                              mc.beta, W_U, W_G, st);
      st = wstage<kRannacher, R>(memo_r, W, P, n, nocache, flo, fhi, o.bc_left, right_bc(o, t_next),
                              mc.alpha, mc.beta, W_G, W_U, st);
      step = 1;
      if (o.nt >= 1) record(1, W_U);
    }
    for (; step < o.nt && st == kStatusOk; ++step) {
      const double tt = static_cast<double>(step) * dt;
      const double t1 = tt + mc.gamma * dt;
      const double tn = static_cast<double>(step + 1) * dt;
      const bool last = (step == o.nt - 1);
      st = wstage<kStage1, R>(memo1, W, P, n, nocache, flo, fhi, o.bc_left, right_bc(o, t1), mc.alpha,
                           mc.beta, W_U, W_G, st);
      st = wstage<kStage2, R>(memo2, W, P, n, nocache, flo, fhi, o.bc_left, right_bc(o, tn), mc.alpha,
                           mc.beta, W_G, last ? W_G : W_U, st);
      if (sc) record(step + 1, last ? W_G : W_U);
    }
    // the solution back into the tile rows for outputs_kernel
    for (int r = 0; r < R; ++r) {
      const int i = lane * R + r;
      if (i >= n) continue;
      double* p = P.rp(i);
      p[A_U * kTile] = W.atl(W_U, r, lane);
      p[A_G * kTile] = W.atl(W_G, r, lane);
    }
    if (lane == 0) status[k] = st;
    __syncwarp();
  }
}

// Concrete kernels, one per row count (a __global__ template is not used).
#define MGPU_WMARCH_KERNEL(RT)                                                                   \
  __global__ void __launch_bounds__(32) wmarch_kernel_##RT(                                     \
      const TileDev* __restrict__ tiles, const int32_t* __restrict__ wt, int nwt,               \
      const OptDev* __restrict__ opts, double* __restrict__ pool,                               \
      const uint8_t* __restrict__ flags, const int32_t* __restrict__ mode,                      \
      int32_t* __restrict__ status, int* __restrict__ queue, MarchConst mc) {                   \
    extern __shared__ double wsm[];                                                             \
    wmarch_body<RT>(wsm, tiles, wt, nwt, opts, pool, flags, mode, status, queue, mc);           \
  }
MGPU_WMARCH_KERNEL(1)
MGPU_WMARCH_KERNEL(2)
MGPU_WMARCH_KERNEL(4)
MGPU_WMARCH_KERNEL(8)
MGPU_WMARCH_KERNEL(16)
MGPU_WMARCH_KERNEL(32)
#undef MGPU_WMARCH_KERNEL

// ------------------------------------------------------------------- host --

size_t wmarch_smem_bytes(int R) {
  return sizeof(double) * static_cast<size_t>(kWArrays) * R * 32 + static_cast<size_t>(R) * 32;
}

int wmarch_rows_per_lane(int n) {
  // the instantiated row counts: 1, 2, 4, 8, 16, 32 rows per lane
  int R = 1;
  while (R * 32 < n) R *= 2;
  return R;
}

int wmarch_max_rows() { return 32; }

namespace {
using WmarchFn = void (*)(const TileDev*, const int32_t*, int, const OptDev*, double*,
                          const uint8_t*, const int32_t*, int32_t*, int*, MarchConst);
WmarchFn wmarch_kernel_for(int R) {
  switch (R) {
    case 1: return wmarch_kernel_1;
    case 2: return wmarch_kernel_2;
    case 4: return wmarch_kernel_4;
    case 8: return wmarch_kernel_8;
    case 16: return wmarch_kernel_16;
    default: return wmarch_kernel_32;
  }
}
// Opt each kernel in to its dynamic shared memory once per process (the
// attribute applies on every device the kernel runs on).
void wmarch_opt_in() {
  static bool done = false;
  if (done) return;
  for (int R = 1; R <= 32; R *= 2)
    check(cudaFuncSetAttribute(reinterpret_cast<const void*>(wmarch_kernel_for(R)),
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(wmarch_smem_bytes(R))),
          "wmarch smem attribute");
  done = true;
}
}  // namespace

void wmarch_launch(void* stream, int num_sms, const TileDev* tiles, const int32_t* wt, int nwt,
                   const OptDev* opts, double* pool, const uint8_t* flags, const int32_t* mode,
                   int32_t* status, int* queue, const MarchConst& mc, int R, int max_blocks) {
  if (nwt <= 0) return;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t smem = wmarch_smem_bytes(R);
  wmarch_opt_in();
  const WmarchFn fn = wmarch_kernel_for(R);
  int bps = 0;
  check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fn, 32, smem), "occupancy");
  int blocks = std::max(1, std::min(num_sms * std::max(bps, 1), nwt * kTile));
  if (max_blocks > 0) blocks = std::min(blocks, max_blocks);
  fn<<<blocks, 32, smem, st>>>(tiles, wt, nwt, opts, pool, flags, mode, status, queue, mc);
  check(cudaGetLastError(), "wmarch_kernel launch");
}

WarpPlan plan_warp_tiles(const TileDev* tiles, int ntiles, int tv_tile0, int num_sms,
                         double thread_scale) {
  WarpPlan plan;
  plan.flag.assign(static_cast<size_t>(std::max(ntiles, 0)), 0);
  int force = -1;
  if (const char* e = std::getenv("MANGO_GPU_WARP_MARCH")) force = std::atoi(e) != 0 ? 1 : 0;
  if (force == 0 || ntiles <= 0) return plan;
  const int rmax = wmarch_max_rows();
  int64_t options = 0;
  int R = 1;
  const int last = std::min(ntiles, tv_tile0);
  for (int t = 0; t < last; ++t) {
    const int r = wmarch_rows_per_lane(tiles[t].nx);
    if (r > rmax) continue;
    options += tiles[t].count;
    R = std::max(R, r);
  }
  if (options == 0) return plan;
  wmarch_opt_in();
  int bps = 0;
  check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, wmarch_kernel_for(R), 32,
                                                      wmarch_smem_bytes(R)),
        "occupancy");
  const int64_t wave = static_cast<int64_t>(num_sms) * std::max(bps, 1);
  // Cost model of the two layouts for the candidate tiles, in microseconds,
  // from measurements on GB300 (101 x 498 and 201 x 1000 grids, 200 to
  // 65,536 options, both layouts forced): the warp march takes about
  // kWarpStepUs + kWarpStepUsPerR * R per time step and wave of resident
  // warps; the thread march about kThreadRowUs per row and step for a tile
  // whose warp has its sub-partition to itself, or, once the tiles crowd the
  // sub-partitions, kThreadRowTileUs per row, step and tile overall.
  constexpr double kWarpStepUs = 10.8, kWarpStepUsPerR = 3.47;
  constexpr double kThreadRowUs = 1.0, kThreadRowTileUs = 0.93e-3;
  int rows = 0, steps = 0;
  for (int t = 0; t < last; ++t)
    if (wmarch_rows_per_lane(tiles[t].nx) <= rmax) {
      rows = std::max(rows, tiles[t].nx);
      steps = std::max(steps, tiles[t].nt);
    }
  const double waves = static_cast<double>((options + wave - 1) / wave);
  const double warp_us = steps * (kWarpStepUs + kWarpStepUsPerR * R) * waves;
  const double thread_us = thread_scale * steps *
                           std::max(rows * kThreadRowUs, static_cast<double>(last) * rows * kThreadRowTileUs);
  if (force == 1 || warp_us < thread_us) {
    for (int t = 0; t < last; ++t)
      if (wmarch_rows_per_lane(tiles[t].nx) <= rmax) {
        plan.tiles.push_back(t);
        plan.flag[t] = 1;
      }
    plan.R = R;
    return plan;
  }
  // A large batch: only the long poles, when the tile costs (rows x steps of
  // the tile's widest and longest lane) are uneven.
  int64_t cap = kLongWarpOptions;
  if (const char* e = std::getenv("MANGO_GPU_WARP_LONG")) cap = std::atoll(e);
  if (cap <= 0) return plan;
  std::vector<std::pair<double, int>> cost;
  double sum = 0.0;
  for (int t = 0; t < last; ++t) {
    const double c = static_cast<double>(tiles[t].nx) * tiles[t].nt;
    sum += c;
    if (wmarch_rows_per_lane(tiles[t].nx) <= rmax) cost.push_back({c, t});
  }
  const double mean = sum / std::max(last, 1);
  std::sort(cost.begin(), cost.end(), [](const auto& a, const auto& b) { return a.first > b.first; });
  int64_t taken = 0;
  int Rw = 1;
  for (const auto& [c, t] : cost) {
    if (c <= 2.0 * mean || taken + tiles[t].count > cap) break;
    plan.flag[t] = 1;
    taken += tiles[t].count;
    Rw = std::max(Rw, wmarch_rows_per_lane(tiles[t].nx));
  }
  if (taken == 0) return plan;
  for (int t = 0; t < last; ++t)
    if (plan.flag[t]) plan.tiles.push_back(t);
  plan.R = Rw;
  plan.concurrent = true;
  plan.blocks = 2 * num_sms;
  return plan;
}

}  // namespace mgpu
