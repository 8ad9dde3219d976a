// noalloc.cu -- batched American pricing without any device allocation.
//
// Why: some callers cannot allocate GPU memory at the moment they need a
// price -- e.g. code running under an allocator that owns the whole device
// (a framework's caching pool that must not be fragmented), code inside a
// region where cudaMalloc is forbidden or would serialise the device, or
// embedded callers with a fixed memory budget.  For them,
// mango_gpu_price_american_batch_noalloc prices a bounded batch using one
// file-scope device array that every GPU loading this library holds until
// the process exits.  It calls no cudaMalloc/cudaFree/cudaMallocAsync and no
// allocating library routine.
//
// Limits (the array is sized for them, ~32 MB of device memory per GPU):
//   at most kNoAllocMaxOptions options per call, and at most
//   kNoAllocMaxRows grid rows in total, counted as the sum over 32-option
//   tiles (options sorted by grid size) of 32 x the tile's largest n_space.
// Larger requests are rejected with MANGO_ERR_VALIDATION and a message.
//
// Set-up: the first call on a device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress; make that first call
// outside any stream capture.  The calling thread's current device is the
// same after the call as before it.  A call that fails as a whole (a limit,
// a CUDA error) still writes every slot: NaN results and the call's status.  Every call shares the array and the static
// host staging buffers: calls are serialised on the host by a mutex, but two
// calls whose GPU work overlaps (different streams) race on the array, so
// order them on one stream or synchronise between them.  Whatever must start
// at zero (the work-queue counter) is cleared on every call; everything else
// is fully rewritten before it is read.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "grid_host.hpp"
#include "march.cuh"
#include "mango_gpu.h"

namespace mgpu {

__global__ void prep_kernel(const TileDev*, int, const OptDev*, const double*, double*, uint8_t*,
                            int32_t*, MarchConst);
__global__ void march_kernel(const TileDev*, int, const OptDev*, double*, const uint8_t*,
                             const int32_t*, int32_t*, int*, MarchConst);
__global__ void outputs_kernel(const TileDev*, int, const OptDev*, const double*, double*,
                               const int32_t*, const int32_t*, MarchConst, double*);

namespace noalloc {

constexpr int64_t kMaxOptions = 4096;
constexpr int64_t kMaxRows = 131072;
constexpr int64_t kMaxTiles = kMaxOptions / kTile;
constexpr int64_t kMaxSpace = kMaxRows / kTile;  // largest n_space a single tile can hold

// Byte offsets of the regions inside the scratch array (all 256-aligned).
constexpr size_t align256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t kOffPool = 0;
constexpr size_t kOffXs = align256(kOffPool + sizeof(double) * A_COUNT * kMaxRows);
constexpr size_t kOffOut4 = align256(kOffXs + sizeof(double) * kMaxRows);
constexpr size_t kOffFlags = align256(kOffOut4 + sizeof(double) * 4 * kMaxOptions);
constexpr size_t kOffMode = align256(kOffFlags + kMaxRows);
constexpr size_t kOffStatus = align256(kOffMode + sizeof(int32_t) * kMaxOptions);
constexpr size_t kOffQueue = align256(kOffStatus + sizeof(int32_t) * kMaxOptions);
constexpr size_t kOffOpts = align256(kOffQueue + sizeof(int32_t) * 4);
constexpr size_t kOffTiles = align256(kOffOpts + sizeof(OptDev) * kMaxOptions);
constexpr size_t kScratchBytes = align256(kOffTiles + sizeof(TileDev) * kMaxTiles);

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Host-side staging, also static (no heap use on this path).
struct HostStage {
  GridSpec spec[kMaxOptions];
  int64_t nt[kMaxOptions];
  int32_t status[kMaxOptions];
  const char* msg[kMaxOptions];
  int32_t order[kMaxOptions];
  TileDev tiles[kMaxTiles];
  OptDev opts[kMaxOptions];
  double xs[kMaxRows];
  double x[kMaxSpace];
  double scratch[kMaxSpace > 1200 ? kMaxSpace : 1200];
  double out4[4 * kMaxOptions];
  int32_t dstatus[kMaxOptions];
};
static HostStage g_host;
static std::mutex g_mutex;

constexpr int kMaxDevices = 64;
static void* g_scratch_ptr[kMaxDevices] = {};
static int g_num_sms[kMaxDevices] = {};
static int g_blocks_per_sm[kMaxDevices] = {};

const char* validate_params(const MangoPricingParams& p) {
  // validate_pricing_params (src/option/option_spec.cpp:8-40, 117-157)
  if (!(p.spot > 0.0) || !std::isfinite(p.spot)) return "invalid spot";
  if (!(p.strike > 0.0) || !std::isfinite(p.strike)) return "invalid strike";
  if (!(p.maturity > 0.0) || !std::isfinite(p.maturity)) return "invalid maturity";
  if (!std::isfinite(p.rate_const)) return "invalid rate";
  if (p.dividend_yield < 0.0 || !std::isfinite(p.dividend_yield)) return "invalid dividend yield";
  if (!(p.volatility > 0.0) || !std::isfinite(p.volatility)) return "invalid volatility";
  if (p.option_type != MANGO_PUT && p.option_type != MANGO_CALL) return "invalid option type";
  if (p.n_tenor_points != 0) return "yield curves are not supported by the no-allocation entry point";
  if (p.n_dividends != 0) return "discrete dividends are not supported by the no-allocation entry point";
  return nullptr;
}

// resolve_grid (src/option/american_option.cpp:54-73) into static storage.
const char* resolve_grid(const MangoPricingParams& p, const MangoGpuGrid& g, GridSpec* spec,
                         int64_t* nt) {
  const Accuracy def = default_accuracy();
  switch (g.kind) {
    case MANGO_GPU_GRID_AUTO:
    case MANGO_GPU_GRID_FIXED_N:
    case MANGO_GPU_GRID_FIXED_N_AT_VOL: {
      Accuracy a = def;
      const bool pinned = g.kind != MANGO_GPU_GRID_AUTO;
      if (pinned) {
        if (g.n_space < 3 || g.n_time < 0) return "grid: n_space >= 3 and n_time >= 0 required";
        if (g.n_space > kMaxSpace) return "grid: n_space above the no-allocation limit";
        a.min_points = a.max_points = g.n_space;
      }
      // FIXED_N_AT_VOL sizes the grid at the volatility in g.alpha instead
      // of the option's own, as the allocating batch does.
      const double vol = g.kind == MANGO_GPU_GRID_FIXED_N_AT_VOL ? g.alpha : p.volatility;
      if (!(vol > 0.0) || !std::isfinite(vol)) return "grid: sizing volatility must be > 0";
      int64_t nt_auto = 0;
      estimate_grid(p.spot, p.strike, p.maturity, vol, a, spec, &nt_auto, g_host.scratch,
                    static_cast<int64_t>(sizeof(g_host.scratch) / sizeof(double)));
      if (spec->n > kMaxSpace) return "grid: n_space above the no-allocation limit";
      *nt = (pinned && g.n_time > 0) ? g.n_time : nt_auto;
      break;
    }
    case MANGO_GPU_GRID_SINH:
      if (g.n_space < 3 || g.n_time < 1) return "grid: n_space >= 3 and n_time >= 1 required";
      if (!(g.x_min < g.x_max)) return "grid: x_min < x_max required";
      if (!(g.alpha > 0.0)) return "grid: alpha > 0 required";
      *spec = sinh_spec(g.x_min, g.x_max, g.n_space, g.alpha);
      *nt = g.n_time;
      break;
    case MANGO_GPU_GRID_UNIFORM:
      if (g.n_space < 3 || g.n_time < 1) return "grid: n_space >= 3 and n_time >= 1 required";
      if (!(g.x_min < g.x_max)) return "grid: x_min < x_max required";
      *spec = uniform_spec(g.x_min, g.x_max, g.n_space);
      *nt = g.n_time;
      break;
    default:
      return "grid: unknown kind";
  }
  if (spec->n > kMaxSpace) return "grid: n_space above the no-allocation limit";
  if (*nt > 100000000) return "grid: n_time above 1e8";
  return nullptr;
}

void set_err(MangoError* err, int32_t code, const char* msg) {
  if (!err) return;
  err->code = code;
  std::snprintf(err->message, sizeof(err->message), "%s", msg);
}

bool cuda_ok(cudaError_t e, const char* what, MangoError* err) {
  if (e == cudaSuccess) return true;
  if (err) {
    err->code = MANGO_ERR_SOLVER;
    std::snprintf(err->message, sizeof(err->message), "%s: %s", what, cudaGetErrorString(e));
  }
  return false;
}

// Every slot NaN with one status: a call that fails as a whole never leaves
// the caller's slots holding stale results.
void fail_all(MangoGpuAmericanOut* out, uint64_t n, int32_t status, uint64_t* out_failed) {
  for (uint64_t i = 0; i < n; ++i) {
    MangoGpuAmericanOut& o = out[i];
    o.value = o.delta = o.gamma = o.theta = NAN;
    o.status = status;
    o.n_space = o.n_time = 0;
    o.reserved = 0;
  }
  if (out_failed) *out_failed = n;
}

// Restores the calling thread's current device on every return path.
struct DeviceGuard {
  int prev = -1;
  DeviceGuard() {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace noalloc
}  // namespace mgpu

using namespace mgpu;
using namespace mgpu::noalloc;

extern "C" MangoStatus mango_gpu_price_american_batch_noalloc(
    int32_t device, void* stream, const MangoPricingParams* params, uint64_t n,
    const MangoGpuGrid* grids, uint64_t grid_stride, const MangoGpuTrbdf2* trbdf2,
    MangoGpuAmericanOut* out, uint64_t* out_failed, MangoError* err) {
  if (n > 0 && (!params || !out)) {
    set_err(err, MANGO_ERR_VALIDATION, "null params or out");
    return MANGO_ERR_VALIDATION;
  }
  if (n > static_cast<uint64_t>(kMaxOptions)) {
    set_err(err, MANGO_ERR_VALIDATION,
            "no-allocation entry point: more than 4096 options in one call");
    fail_all(out, n, MANGO_ERR_VALIDATION, out_failed);
    return MANGO_ERR_VALIDATION;
  }
  if (device < 0 || device >= kMaxDevices) {
    set_err(err, MANGO_ERR_VALIDATION, "invalid device index");
    fail_all(out, n, MANGO_ERR_VALIDATION, out_failed);
    return MANGO_ERR_VALIDATION;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  const DeviceGuard device_guard;
  auto cuda_fail = [&]() {
    fail_all(out, n, MANGO_ERR_SOLVER, out_failed);
    return MANGO_ERR_SOLVER;
  };
  if (!cuda_ok(cudaSetDevice(device), "cudaSetDevice", err)) return cuda_fail();
  // Once per device, with that device current: the array's device address.
  if (!g_scratch_ptr[device]) {
    void* ptr = nullptr;
    if (!cuda_ok(cudaGetSymbolAddress(&ptr, g_scratch), "cudaGetSymbolAddress", err))
      return cuda_fail();
    int sms = 0, bps = 0;
    if (!cuda_ok(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device),
                 "cudaDeviceGetAttribute", err))
      return cuda_fail();
    if (!cuda_ok(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, march_kernel, 128, 0),
                 "occupancy", err))
      return cuda_fail();
    g_num_sms[device] = sms;
    g_blocks_per_sm[device] = std::max(1, bps);
    g_scratch_ptr[device] = ptr;
  }
  unsigned char* base = static_cast<unsigned char*>(g_scratch_ptr[device]);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  HostStage& H = g_host;

  MarchConst mc{};
  mc.gamma = (trbdf2 && trbdf2->gamma > 0.0) ? trbdf2->gamma : 2.0 - std::sqrt(2.0);
  mc.rannacher = trbdf2 ? (trbdf2->rannacher_startup != 0) : 1;
  {
    const double omg = 1.0 - mc.gamma, tmg = 2.0 - mc.gamma, den = mc.gamma * tmg;
    mc.alpha = 1.0 / den;
    mc.beta = -(omg * omg) / den;
  }

  const int64_t nn = static_cast<int64_t>(n);
  int64_t m = 0;
  for (int64_t i = 0; i < nn; ++i) {
    const char* msg = validate_params(params[i]);
    if (!msg) {
      MangoGpuGrid g{};
      g.kind = MANGO_GPU_GRID_AUTO;
      if (grids) g = grids[grid_stride ? i : 0];
      msg = resolve_grid(params[i], g, &H.spec[i], &H.nt[i]);
    }
    H.msg[i] = msg;
    H.status[i] = msg ? MANGO_ERR_VALIDATION : MANGO_OK;
    if (!msg) H.order[m++] = static_cast<int32_t>(i);
  }
  std::sort(H.order, H.order + m, [&](int32_t a, int32_t c) {
    if (H.spec[a].n != H.spec[c].n) return H.spec[a].n > H.spec[c].n;
    if (H.nt[a] != H.nt[c]) return H.nt[a] > H.nt[c];
    return a < c;
  });
  const int32_t ntiles = static_cast<int32_t>((m + kTile - 1) / kTile);
  int64_t rows = 0;
  for (int32_t t = 0; t < ntiles; ++t) {
    TileDev& td = H.tiles[t];
    td.first = t * kTile;
    td.count = static_cast<int32_t>(std::min<int64_t>(kTile, m - td.first));
    int64_t nx = 0, ntm = 0;
    for (int l = 0; l < td.count; ++l) {
      const int32_t s = H.order[td.first + l];
      nx = std::max<int64_t>(nx, H.spec[s].n);
      ntm = std::max<int64_t>(ntm, H.nt[s]);
    }
    td.nx = static_cast<int32_t>(nx);
    td.nt = static_cast<int32_t>(ntm);
    td.off = static_cast<int64_t>(A_COUNT) * rows;
    td.xoff = rows;
    td.foff = rows;
    rows += nx * kTile;
  }
  if (rows > kMaxRows) {
    set_err(err, MANGO_ERR_VALIDATION,
            "no-allocation entry point: batch needs more than 131072 grid rows");
    fail_all(out, n, MANGO_ERR_VALIDATION, out_failed);
    return MANGO_ERR_VALIDATION;
  }
  for (int32_t t = 0; t < ntiles; ++t) {
    const TileDev& td = H.tiles[t];
    for (int l = 0; l < kTile; ++l) {
      double* dst = H.xs + td.xoff + l;
      if (l >= td.count) {
        for (int i = 0; i < td.nx; ++i) dst[static_cast<size_t>(i) * kTile] = 0.0;
        continue;
      }
      const int32_t s = H.order[td.first + l];
      const GridSpec& sp = H.spec[s];
      const MangoPricingParams& p = params[s];
      generate_grid(sp, H.x);
      for (int i = 0; i < td.nx; ++i)
        dst[static_cast<size_t>(i) * kTile] = H.x[std::min<int64_t>(i, sp.n - 1)];
      OptDev& o = H.opts[td.first + l];
      o.dt = (p.maturity - 0.0) / static_cast<double>(H.nt[s]);
      o.sigma = p.volatility;
      o.r = p.rate_const;
      o.q = p.dividend_yield;
      const bool put = p.option_type == MANGO_PUT;
      o.bc_left = put ? std::max(1.0 - std::exp(H.x[0]), 0.0) : 0.0;
      o.exp_xr = std::exp(H.x[sp.n - 1]);
      o.x_spot = std::log(p.spot / p.strike);
      o.spot = p.spot;
      o.strike = p.strike;
      o.n = static_cast<int32_t>(sp.n);
      o.nt = static_cast<int32_t>(H.nt[s]);
      o.is_put = put ? 1 : 0;
      o.orig = s;
    }
  }

  if (m > 0) {
    double* d_pool = reinterpret_cast<double*>(base + kOffPool);
    double* d_xs = reinterpret_cast<double*>(base + kOffXs);
    double* d_out4 = reinterpret_cast<double*>(base + kOffOut4);
    uint8_t* d_flags = reinterpret_cast<uint8_t*>(base + kOffFlags);
    int32_t* d_mode = reinterpret_cast<int32_t*>(base + kOffMode);
    int32_t* d_status = reinterpret_cast<int32_t*>(base + kOffStatus);
    int* d_queue = reinterpret_cast<int*>(base + kOffQueue);
    OptDev* d_opts = reinterpret_cast<OptDev*>(base + kOffOpts);
    TileDev* d_tiles = reinterpret_cast<TileDev*>(base + kOffTiles);
    if (!cuda_ok(cudaMemcpyAsync(d_xs, H.xs, sizeof(double) * rows, cudaMemcpyHostToDevice, st),
                 "H2D grids", err) ||
        !cuda_ok(cudaMemcpyAsync(d_opts, H.opts, sizeof(OptDev) * m, cudaMemcpyHostToDevice, st),
                 "H2D options", err) ||
        !cuda_ok(cudaMemcpyAsync(d_tiles, H.tiles, sizeof(TileDev) * ntiles,
                                 cudaMemcpyHostToDevice, st),
                 "H2D tiles", err) ||
        !cuda_ok(cudaMemsetAsync(d_queue, 0, sizeof(int32_t) * 4, st), "clear queue", err))
      return cuda_fail();
    const int threads = ntiles * kTile;
    prep_kernel<<<(threads + 127) / 128, 128, 0, st>>>(d_tiles, ntiles, d_opts, d_xs, d_pool,
                                                       d_flags, d_mode, mc);
    const int blocks = std::max(1, std::min<int>(g_num_sms[device] * g_blocks_per_sm[device],
                                                 (ntiles + 3) / 4));
    march_kernel<<<blocks, 128, 0, st>>>(d_tiles, ntiles, d_opts, d_pool, d_flags, d_mode,
                                         d_status, d_queue, mc);
    outputs_kernel<<<(threads + 127) / 128, 128, 0, st>>>(d_tiles, ntiles, d_opts, d_xs, d_pool,
                                                          d_mode, d_status, mc, d_out4);
    if (!cuda_ok(cudaGetLastError(), "kernel launch", err) ||
        !cuda_ok(cudaMemcpyAsync(H.out4, d_out4, sizeof(double) * 4 * m, cudaMemcpyDeviceToHost,
                                 st),
                 "D2H results", err) ||
        !cuda_ok(cudaMemcpyAsync(H.dstatus, d_status, sizeof(int32_t) * m,
                                 cudaMemcpyDeviceToHost, st),
                 "D2H status", err) ||
        !cuda_ok(cudaStreamSynchronize(st), "stream synchronize", err))
      return cuda_fail();
  }

  uint64_t failed = 0;
  const char* first = nullptr;
  for (int64_t i = 0; i < nn; ++i) {
    MangoGpuAmericanOut& o = out[i];
    o.value = o.delta = o.gamma = o.theta = NAN;
    o.status = H.status[i];
    o.n_space = static_cast<int32_t>(H.status[i] == MANGO_OK ? H.spec[i].n : 0);
    o.n_time = static_cast<int32_t>(H.status[i] == MANGO_OK ? H.nt[i] : 0);
    o.reserved = 0;
    if (H.msg[i] && !first) first = H.msg[i];
  }
  for (int64_t k = 0; k < m; ++k) {
    MangoGpuAmericanOut& o = out[H.order[k]];
    o.status = H.dstatus[k];
    o.value = H.out4[4 * k + 0];
    o.delta = H.out4[4 * k + 1];
    o.gamma = H.out4[4 * k + 2];
    o.theta = H.out4[4 * k + 3];
  }
  for (int64_t i = 0; i < nn; ++i) failed += out[i].status != MANGO_OK;
  if (out_failed) *out_failed = failed;
  if (failed && err) set_err(err, MANGO_OK, first ? first : "solver failure");
  return MANGO_OK;
}
