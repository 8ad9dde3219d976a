// march_tan.cuh -- layout of the tangent pool of march_tan.cu and the host
// entry points that run the tangent march on a batch.
#pragma once
#include <cstdint>

#include "march.cuh"

namespace mgpu {

// Directions a tangent march differentiates along.
constexpr int32_t kDirSigma = 0;
constexpr int32_t kDirRate = 1;
constexpr int32_t kDirDividend = 2;

// Per row, per direction, the arrays of the tangent pool.
enum TanArray : int {
  T_E1L = 0,  // d/dtheta of the pre-scaled stage-1 stencil (cached rows)
  T_E1D,
  T_E1U,
  T_N1H,      // d/dtheta of -(l1 / pivot1)
  T_NC1,      // d/dtheta of -c'1 (cached)
  T_A2H,      // d/dtheta of alpha / pivot2
  T_B2H,      // d/dtheta of beta / pivot2
  T_N2H,      // d/dtheta of -(l2 / pivot2)
  T_NC2,      // d/dtheta of -c'2 (cached)
  T_JL,       // d/dtheta of the Jacobian row (rows off the cache:
  T_JD,       //   band derivative = -w x these)
  T_JU,
  T_U,        // tangent of u^n
  T_G,        // tangent of u^{n+gamma} (and of the final u)
  T_D,        // tangent of the Thomas d'
  T_CP,       // -d/dtheta c' of rows solved off the cache
  T_COUNT
};

// Doubles per sorted option in the output of outputs_tan_kernel:
// value, delta, dV/dK, then one derivative per direction.
constexpr int tan_out_stride(int nd) { return 3 + nd; }

struct TanConst {
  int32_t dirs[3];  // direction of tangent j (kDir*)
  int32_t pad;
};

// Offset (doubles) of a tile's tangent block: the tangent pool keeps the
// primal pool's row order with ND * T_COUNT arrays per row.
template <int ND>
__host__ __device__ __forceinline__ int64_t tan_off(const TileDev& td) {
  return td.off / A_COUNT * (ND * T_COUNT);
}

#ifdef __CUDACC__
template <int ND>
struct TanView {
  double* B;  // tile block + lane
  __device__ __forceinline__ double& at(int j, int a, int i) const {
    return B[((static_cast<size_t>(i) * ND + j) * T_COUNT + a) * kTile];
  }
};

#endif

// Host: launch setup, tangent setup, tangent march and tangent outputs for
// the tiles of a packed batch on stream st (the caller clears queue[0]).
// tpool must hold tan_pool_doubles(nd, primal pool doubles); out
// tan_out_stride(nd) doubles per sorted option.  nd is 1 or 3.
int64_t tan_pool_doubles(int nd, int64_t pool_doubles);
void tan_launch(int nd, void* stream, int num_sms, const TileDev* tiles, int ntiles,
                const OptDev* opts, const double* xs, double* pool, double* tpool,
                uint8_t* flags, int32_t* mode, int32_t* status, int* queue, const TanConst& tc,
                const MarchConst& mc, double* out);

}  // namespace mgpu
