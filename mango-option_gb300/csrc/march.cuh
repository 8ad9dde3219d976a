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
  A_CP,       // Thomas c' of rows solved off the cache
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
};

// Status codes written per option (MangoStatus values).
constexpr int32_t kStatusOk = 0;
constexpr int32_t kStatusSolver = 5;

}  // namespace mgpu
