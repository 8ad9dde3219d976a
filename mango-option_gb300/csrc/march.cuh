// march.cuh -- device data layout shared by the American-option kernels.
//
// Options are sorted by (n_space, n_time) descending and packed into tiles
// of 32: one warp marches one tile, one lane per option (thread-per-option
// Thomas sweeps; the tridiagonal recurrences are serial along the grid, so
// the work-optimal parallel axis is across options).
#pragma once
#include <cstdint>

namespace mgpu {

constexpr int kTile = 32;

// Per-row arrays of a tile block, laid out [row][array][lane]: one warp
// touching array a of row i reads 32 consecutive doubles (two 128-byte
// lines), and every array of a row is reached from one row pointer with an
// immediate offset.  The arrays read in every time step come first.
enum TileArray : int {
  A_E1L = 0,  // stage-1 right-hand-side stencil pre-scaled by the cached
  A_E1D,      //   inverse pivot: d'_i = e_l u_{i-1} + e_d u_i + e_u u_{i+1}
  A_E1U,      //   + n1h d'_{i-1}
  A_N1H,      // stage 1: -(sub-diagonal x cached inverse pivot)
  A_NC1,      // stage 1: -c'_i of the unlocked matrix (cached factor)
  A_PSI,      // obstacle psi = payoff (time invariant for these payoffs)
  A_A2H,      // stage 2: alpha x inverse pivot
  A_B2H,      // stage 2: beta x inverse pivot
  A_N2H,      // stage 2: -(sub-diagonal x inverse pivot)
  A_NC2,      // stage 2: -c'_i (cached)
  A_U,        // state u^n
  A_G,        // state u^{n+gamma} (and the final u)
  A_D,        // Thomas d' scratch
  A_CP,       // Thomas -c' of rows solved off the cache (stage 1, Rannacher)
  A_CP2,      // the same for stage 2
  A_IP1,      // inverse pivot of stage-1 rows solved off the cache
  A_IP2,      // the same for stage 2
  A_E1L0,     // unscaled stage-1 stencil (rows off the cache)
  A_E1D0,
  A_E1U0,
  A_L1, A_D1, A_U1,  // stage-1 matrix bands (assemble_jacobian form)
  A_L2, A_D2, A_U2,  // stage-2 matrix bands
  A_LR, A_DR, A_UR,  // Rannacher half-step bands
  A_COUNT
};
constexpr int kRowStride = A_COUNT * 32;  // doubles between consecutive rows

// Per-option parameters, in sorted order.
struct OptDev {
  double dt;
  double sigma, r, q;
  double bc_left;   // put: max(1 - e^{x_0}, 0); call: 0
  double exp_xr;    // call: e^{x_{n-1}} (right boundary e^{x} - e^{-r t})
  double x_spot;    // ln(S/K)
  double spot, strike;
  int32_t n, nt;
  int32_t is_put;
  int32_t orig;     // index in the caller's array
};

// One option's grid (GridSpec of grid_host.hpp as plain data), generated on
// the device by grid_kernel / grid_finish_kernel with generate_grid's
// formulas (GridSpec::generate, src/pde/core/grid.hpp:364-498).
struct GridDev {
  int32_t type;        // GridSpec::Type
  int32_t n_clusters;
  int32_t n;
  int32_t pad;
  double x_min, x_max, concentration;
  double c_center[4], c_alpha[4], c_weight[4];
};

struct TileDev {
  int64_t off;      // offset (doubles) of this tile's block in the pool
  int64_t xoff;     // offset (doubles) of this tile's grid in the grid array
  int64_t foff;     // offset (bytes) of this tile's lock-candidate flags
  int32_t nx;       // rows (max n_space over the tile's lanes)
  int32_t nt;       // max n_time over the tile's lanes
  int32_t first;    // first sorted option index
  int32_t count;    // lanes in use (<= 32)
};

struct MarchConst {
  double gamma;     // TR-BDF2 gamma
  double alpha;     // 1 / (gamma (2 - gamma))
  double beta;      // -(1 - gamma)^2 / (gamma (2 - gamma))
  int32_t rannacher;
  int32_t value_only;            // outputs: skip delta/gamma/theta
  const double* sigma;           // per-option volatility override (sorted), or null
  const int32_t* active;         // per-option run flag (sorted), or null = all
  // Snapshot taps (Grid::record, src/pde/core/grid.hpp:947-961), or null:
  // per sorted option, snap_count ascending state indices starting at
  // snap_idx + snap_begin[k]; the state after that step goes to
  // snap_out + snap_off[k] + j * n.
  const int32_t* snap_idx;
  const int32_t* snap_begin;
  const int32_t* snap_count;
  const int64_t* snap_off;
  double* snap_out;
  // Sorted index of the first option on the time-varying march
  // (march_tv.cu); options from here on are skipped by prep and march.
  int32_t tv_first = 0x7fffffff;
  // Per tile, nonzero: the tile's options are marched one warp per option
  // (wmarch.cu) and march_kernel skips it; null: every tile on march_kernel.
  const uint8_t* tile_warp = nullptr;
  // Test hook (set by the host from MANGO_GPU_SINGULAR_PIVOT): sorted index
  // of the one option whose row-1 diagonals prep_kernel zeroes, so that its
  // first pivot is exactly 0 and the solve reports kStatusSolver as a
  // singular Thomas pivot does; -1 = none.
  int32_t singular_pivot = -1;
  // Tiles assigned to SM sub-partitions (uneven batches), or nbins = 0.  A
  // warp of the binned launch takes the tiles of list (SM index x 4 + warp
  // slot mod 4) in order, marks each in tile_done, and leaves when its list
  // is empty; a second launch (tile_done set, nbins = 0) marches whatever
  // tile no warp took.
  const int32_t* bin_off = nullptr;   // nbins + 1 offsets into bin_tiles
  const int32_t* bin_tiles = nullptr;
  int* bin_cnt = nullptr;             // per list, tiles taken so far
  const int32_t* sm_index = nullptr;  // %smid -> dense SM index, -1: none
  int32_t nsmid = 0;                  // entries of sm_index
  int32_t nbins = 0;
  uint8_t* tile_done = nullptr;
  // Hand-off of a tile's remaining steps (non-binned thread-march launches
  // without snapshots), or ho_ctl = null: a warp whose queue ran dry waits on
  // a claimed slot (ho_ctl[0] counts the claims); a marching warp that sees a
  // claim not yet served (ho_ctl[0] > ho_ctl[1]) takes a slot (ho_ctl[1]),
  // stores its tile and next step there and leaves, so that the tiles of a
  // sub-partition holding four warps end on one holding fewer.  ho_ctl[2]
  // counts the tiles finished or skipped; waiting warps leave once it reaches
  // ntiles.  A tile moves at most once (ho_moved).
  int* ho_ctl = nullptr;
  unsigned long long* ho_slot = nullptr;
  uint8_t* ho_moved = nullptr;
  int32_t ho_cap = 0;
  int32_t ho_total = 0;  // tiles this launch finishes or skips (its ntiles)
};

// Per-option data of the time-varying march, indexed by sorted index minus
// MarchConst::tv_first.  Pairs are stored as two consecutive doubles.
struct TvDev {
  double T;           // maturity: calendar time s = max(0, T - tau)
  double r;           // constant rate when n_curve == 0
  int32_t tp_off;     // first explicit time point in the point array, -1: t_i = i dt
  int32_t curve_off;  // first (tenor, log discount) pair, sorted by tenor
  int32_t n_curve;    // 0: constant rate r
  int32_t ev_off;     // first (tau, amount / strike) dividend event, sorted by tau
  int32_t n_ev;
  int32_t pad;
};

#ifdef __CUDACC__
// Rows of one lane inside a tile block ([row][array][lane]).
struct TileView {
  double* B;  // tile block + lane
  int NX;
  __device__ __forceinline__ double* rp(int i) const {
    return B + static_cast<size_t>(i) * kRowStride;
  }
  __device__ __forceinline__ double& at(int a, int i) const { return rp(i)[a * kTile]; }
};

// [row][lane] arrays (grids, flags).
#define ROW(p, i) (p)[static_cast<size_t>(i) * kTile]

// std::max(a, b) as the reference spells it: (a < b) ? b : a.
__device__ __forceinline__ double dmax_ref(double a, double b) { return (a < b) ? b : a; }

// CubicSpline::find_interval (cubic_spline_solver.hpp:348-368) on a
// [row][lane] grid.
__device__ __forceinline__ int find_interval(const double* __restrict__ X, int n, double xe) {
  if (xe <= ROW(X, 0)) return 0;
  if (xe >= ROW(X, n - 1)) return n - 2;
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = lo + (hi - lo) / 2;
    if (ROW(X, mid) < xe) lo = mid + 1; else hi = mid;
  }
  int idx = lo;
  if (idx > 0 && (idx == n || ROW(X, idx) > xe)) --idx;
  return idx < n - 2 ? idx : n - 2;
}
#endif

// Status codes written per option (MangoStatus values).
constexpr int32_t kStatusOk = 0;
constexpr int32_t kStatusSolver = 5;

}  // namespace mgpu
