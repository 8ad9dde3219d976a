// wmarch.cuh -- host entry points of the warp-per-option march (wmarch.cu).
#pragma once
#include <cstddef>
#include <cstdint>
#include <vector>

#include "march.cuh"

namespace mgpu {

// Shared memory of one warp for options of up to 32 R grid rows.
size_t wmarch_smem_bytes(int R);
// Rows per lane an option of n grid rows needs.
int wmarch_rows_per_lane(int n);
// The largest rows per lane one warp's shared memory holds.
int wmarch_max_rows();
// March the options of the warp tiles wt[0..nwt) (device list of tile
// indices), one warp per option, after prep_kernel; results go back into the
// tile pool for outputs_kernel.  queue[0] must be zero.  R: rows per lane of
// the widest option of those tiles.
void wmarch_launch(void* stream, int num_sms, const TileDev* tiles, const int32_t* wt, int nwt,
                   const OptDev* opts, double* pool, const uint8_t* flags, const int32_t* mode,
                   int32_t* status, int* queue, const MarchConst& mc, int R,
                   int max_blocks = 0);

// Which tiles of a packed set march one warp per option.  The options of the
// tiles [0, ntiles) except the time-varying ones (from tile tv_tile0) are
// candidates when their grid fits a warp's shared memory.  When a measured
// cost model says the warp march finishes them sooner (the last evaluations
// of a batched IV, a table sweep, batches up to a few waves of resident
// warps), every candidate tile goes to the warp march; otherwise the thread
// march keeps them (a full batch keeps every lane busy with its cheaper
// per-row work), except the longest
// tiles of a batch whose tiles differ widely in cost (uneven grids): a
// thread-march warp needs n x n_time dependent row updates for its tile, so
// the tiles of more than twice the mean cost, up to kLongWarpOptions options,
// go to the warp march, which runs beside the thread march on two blocks per
// SM (concurrent = true).  MANGO_GPU_WARP_MARCH = 0 / 1 forces the thread /
// warp layout for the candidates.
struct WarpPlan {
  std::vector<int32_t> tiles;  // warp tiles, ascending
  std::vector<uint8_t> flag;   // per tile: 1 = warp
  int R = 0;                   // rows per lane of the widest warp option
  bool concurrent = false;     // a subset beside the thread march
  int blocks = 0;              // warp-march blocks (0: by occupancy)
};
// thread_scale multiplies the thread march's estimate: 1 for a batch sorted
// by the pricing pipeline, more for working sets whose lanes march slower
// than the model's (the tail of a batched IV).
WarpPlan plan_warp_tiles(const TileDev* tiles, int ntiles, int tv_tile0, int num_sms,
                         double thread_scale = 1.0);

}  // namespace mgpu
