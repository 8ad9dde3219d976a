// engine.hpp -- host side of the GPU engine: the context and resident-batch
// objects behind the C ABI (include/mango_gpu.h), device buffer management
// and the batch pipeline (validate -> grid -> sort/tile -> upload -> setup ->
// march -> outputs -> download).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

#include "grid_host.hpp"
#include "march.cuh"
#include "mango_gpu.h"

namespace mgpu {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

void check(cudaError_t e, const char* what);

// Grow-only device allocation.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  void* get(size_t bytes);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// Grow-only pinned host allocation.
struct HostBuf {
  void* p = nullptr;
  size_t cap = 0;
  void* get(size_t bytes);
  void release();
  template <class T> T* as() const { return static_cast<T*>(p); }
};

// One option after validation and grid resolution, host side.
struct Resolved {
  GridSpec spec;
  int64_t nt = 0;
  int32_t status = 0;  // MangoStatus; non-zero options never reach the GPU
  int32_t orig = 0;
  bool tv = false;         // yield curve or dividends: the time-varying march
  std::vector<double> tp;  // explicit time points (n_time + 1), empty: i * T / n_time
};

// Timings of the last batch call (milliseconds) and work counters.
struct Stats {
  double host_prep_ms = 0, h2d_ms = 0, prep_ms = 0, march_ms = 0, outputs_ms = 0,
         d2h_ms = 0, total_ms = 0;
  int64_t options = 0, tiles = 0, kernel_launches = 0;
  double algo_flops = 0;
  double h2d_bytes = 0, d2h_bytes = 0;
  // FDM IV: quote evaluations on coarse grids with the volatility tangent,
  // and on the own grids
  int64_t iv_evals[2] = {0, 0};
};

// Validation (validate_pricing_params plus the engine's scope) and grid
// resolution; empty string when the option is accepted.
// Yield-curve and dividend checks (YieldCurve::from_points, build_rate,
// build_dividends, the dividend rules of validate_pricing_params); empty
// when accepted.
std::string schedule_error(const MangoTenorPoint* tenor_points, uint64_t n_tenor_points,
                           const MangoDividend* dividends, uint64_t n_dividends, double maturity);
// allow_tv: accept yield curves and discrete dividends (the pricing batch
// entry points); otherwise they are rejected with a message.
std::string validate(const MangoPricingParams& p, bool allow_tv = false);
// The option needs the time-varying march: a yield curve, or a dividend
// strictly inside (0, T).
bool time_varying(const MangoPricingParams& p);
// PDEGridConfig{spec, n_time, dividend times} time domain (resolve_grid).
void explicit_time_domain(double maturity, int64_t n_time, const std::vector<double>& taus,
                          Resolved* r);
std::string resolve(const MangoPricingParams& p, const MangoGpuGrid& g, Resolved* r,
                    std::vector<double>* scratch);

// Run f(i) for i in [0, n) on all host cores, at least grain items per thread.
void parallel_for(int64_t n, const std::function<void(int64_t)>& f, int64_t grain = 512);

void set_err(MangoError* err, int32_t code, const std::string& msg);

// Device buffers of one FDM IV working set (iv.cu), kept per level in the
// context between solves.
constexpr int kIvWorkBufs = 20;

}  // namespace mgpu

struct MangoGpuBatch;

namespace mgpu {
MarchConst make_const(const MangoGpuTrbdf2* trbdf2);
// Validate, resolve grids, sort/tile, pack and upload (batch pipeline).
// reuse: an existing batch whose buffers are refilled (grow-only) instead
// of a new one.
MangoGpuBatch* create_batch(MangoGpuContext* ctx, const MangoPricingParams* params, int64_t n,
                            const MangoGpuGrid* grids, uint64_t grid_stride,
                            const MangoGpuTrbdf2* trbdf2, MangoGpuBatch* reuse = nullptr,
                            cudaStream_t stream = nullptr);
// Same pipeline from already validated and resolved options (res[i].orig
// indexes params; status != 0 entries stay off the device).
MangoGpuBatch* create_batch_resolved(MangoGpuContext* ctx, const MangoPricingParams* params,
                                     std::vector<Resolved> resolved,
                                     std::vector<std::string> messages,
                                     const MangoGpuTrbdf2* trbdf2,
                                     MangoGpuBatch* reuse = nullptr,
                                     cudaStream_t stream = nullptr);
void destroy_batch(MangoGpuBatch* b);
// Deferred grids (MangoGpuBatch::defer_grids): fill the pinned grid array
// and the options' boundary data from the batch's params (host only, any
// thread; the params array must still be alive), then copy both to the
// device on the batch's stream.
void fill_batch_grids(MangoGpuBatch* b);
void upload_batch_grids(MangoGpuBatch* b);
// Enqueue setup, march and outputs (with timing events).
void run_batch(MangoGpuBatch* b);
// Wait, copy results into caller slots, update the context stats.
uint64_t fetch_batch(MangoGpuBatch* b, MangoGpuAmericanOut* out, std::string* first_msg);
// Status of an IV query before any solve, as the reference C ABI reports it
// (iv.cu); msg names the failed check.
int32_t iv_query_status(const MangoIvQuery& q, std::string* msg);

// Price-table sweep (table.cu): argument checks, and the sweep with the
// tensor [m][tau][sigma][r] left in device memory; returns failed slices.
std::string check_table_args(const double* moneyness, uint64_t nm, const double* maturity,
                             uint64_t ntau, const double* volatility, uint64_t nsig,
                             const double* rate, uint64_t nr, double K_ref, double dividend_yield,
                             MangoOptionType option_type);
uint64_t table_sweep_device(MangoGpuContext* ctx, const double* moneyness, uint64_t nm,
                            const double* maturity, uint64_t ntau, const double* volatility,
                            uint64_t nsig, const double* rate, uint64_t nr, double K_ref,
                            double dividend_yield, MangoOptionType option_type,
                            const MangoGpuGrid* grid, double* dten, int64_t* slice_dims);
// Kernels (march.cu).
__global__ void grid_kernel(const TileDev*, const GridDev*, double*);
__global__ void grid_finish_kernel(const TileDev*, int, const GridDev*, double*, OptDev*);
__global__ void prep_kernel(const TileDev*, int, const OptDev*, const double*, double*, uint8_t*,
                            int32_t*, MarchConst);
__global__ void march_kernel(const TileDev*, int, const OptDev*, double*, const uint8_t*,
                             const int32_t*, int32_t*, int*, MarchConst);
__global__ void outputs_kernel(const TileDev*, int, const OptDev*, const double*, double*,
                               const int32_t*, const int32_t*, MarchConst, double*);
// Result functionals of sorted options grp[j] at spot[j] with strike[j]
// (march.cu): the normalized chain's extraction, and value_at.
__global__ void chain_outputs_kernel(int, const int32_t*, const double*, const double*,
                                     const TileDev*, const OptDev*, const double*, double*,
                                     const int32_t*, const int32_t*, MarchConst, double*, int,
                                     double*);
// Time-varying march (march_tv.cu).
__global__ void march_tv_kernel(const TileDev*, int, int, const OptDev*, const TvDev*,
                                const double*, const double*, const double*, const double*,
                                double*, int32_t*, int32_t*, MarchConst);
}  // namespace mgpu

struct MangoGpuContext {
  int device = 0;
  int num_sms = 0;
  int march_blocks_per_sm = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;  // own_stream or a caller's stream
  mgpu::Stats stats;
  // Buffers of the one-shot batch call, kept for the next call (device
  // allocation and host page locking would otherwise be paid every call).
  MangoGpuBatch* scratch = nullptr;
  // Large one-shot batches run as chunks on two streams, so that the host
  // preparation of a chunk overlaps the device work of the one before.
  cudaStream_t aux[2] = {nullptr, nullptr};
  MangoGpuBatch* chunk[2] = {nullptr, nullptr};
  // %smid -> dense SM index (-1: not an SM of this device), probed on first
  // use by a binned launch; nsmid = 0 until then, or when the probe did not
  // see every SM.
  mgpu::DevBuf d_sm_index;
  int nsmid = 0;
  bool sm_probed = false;
  // The price-table sweep's batch and snapshot buffers, kept for the next
  // sweep (a table build calls it once; a caller sweeping repeatedly would
  // otherwise pay some twenty device allocations per call).
  MangoGpuBatch* table_batch = nullptr;
  mgpu::DevBuf table_buf[8];
  // The FDM IV solver's state, kept for the next solve (a fresh solve of
  // 262,144 quotes would otherwise page-lock some 300 MB of host staging
  // and allocate and free several GB of device memory): its two batches
  // (the own grids and Newton's coarse grids, created without march
  // buffers), the per-quote device and pinned host arrays, and the device
  // buffers of the working sets of each level.
  MangoGpuBatch* iv_batch[2] = {nullptr, nullptr};
  mgpu::DevBuf iv_dev[8];
  mgpu::HostBuf iv_host[3];
  mgpu::DevBuf iv_ws[2][mgpu::kIvWorkBufs];
};

struct MangoGpuBatch {
  MangoGpuContext* ctx = nullptr;
  cudaStream_t stream = nullptr;          // all of this batch's device work
  // false: creation leaves the march's pool, flags, modes, statuses and
  // outputs unallocated (the IV batches, whose evaluations march packed
  // working sets of their own)
  bool march_buffers = true;
  // true: the grids are generated on the device from each option's spec
  // (grid_kernel), within a few units in the last place of the host's
  // generate_grid; for grids the reference never sees (the Newton IV
  // method's coarse grids), where the host's sinh evaluations would be
  // most of the preparation
  bool device_grids = false;
  // true: creation leaves the grid points (and the boundary data taken from
  // them) to fill_batch_grids, which may run on another host thread while
  // the device works on something else, and upload_batch_grids (the Newton
  // IV method's own grids, filled during its coarse rounds)
  bool defer_grids = false;
  bool grids_pending = false;              // deferred grids not yet uploaded
  const MangoPricingParams* grid_params = nullptr;  // the params they come from
  int64_t n = 0;                          // caller's slot count
  std::vector<mgpu::Resolved> res;        // per slot
  std::vector<std::string> msgs;          // per slot validation message
  std::vector<int32_t> order;             // sorted position -> slot
  int32_t ntiles = 0;
  mgpu::MarchConst mc{};
  double algo_flops = 0;
  double h2d_bytes = 0;
  double host_prep_ms = 0;
  mgpu::DevBuf d_pool, d_xs, d_grids, d_flags, d_opts, d_tiles, d_mode, d_status, d_out4, d_queue;
  // Time-varying options (sorted last, from mc.tv_first): per-option data,
  // explicit time points, yield-curve pairs, dividend-event pairs.
  mgpu::DevBuf d_tv, d_tv_tp, d_tv_curve, d_tv_ev;
  int32_t tv_tile0 = 0;  // first tile holding a time-varying option
  // Tiles marched one warp per option (wmarch.cu), planned on the first run.
  bool wplan_ready = false;
  int32_t nwt = 0, wR = 0, wblocks = 0;
  bool wconcurrent = false;             // warp march beside the thread march
  cudaStream_t wstream = nullptr;       // its stream, created on first use
  cudaEvent_t wev[2] = {nullptr, nullptr};
  mgpu::DevBuf d_wt, d_tile_warp;
  // Thread-march tiles of an uneven batch assigned to SM sub-partitions
  // (planned with the warp tiles): list offsets then tiles, the list
  // counters, and the per-tile taken flags of the binned launch.
  int32_t nbins = 0;
  mgpu::DevBuf d_bins, d_bin_cnt, d_tile_done;
  mgpu::DevBuf d_handoff;  // the thread march's tile hand-off state (march.cuh)
  mgpu::HostBuf h_xs, h_grids, h_opts, h_tiles, h_out4, h_status;
  cudaEvent_t ev[8] = {};
  bool ran = false;
  // Per-run kernel timing: 4 events per run (before setup, after setup,
  // after march, after outputs), kept for the last kMaxTimedRuns runs.
  static constexpr int kMaxTimedRuns = 256;
  std::vector<cudaEvent_t> run_ev;
  int64_t runs = 0;      // runs since the last timing reset
};
