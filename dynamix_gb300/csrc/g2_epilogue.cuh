// Lag-diagonal sums of a 32 x 32 block of Gram values held one row per lane
// (the tcgen05.ld 32x32b.x32 layout): shared by the tensor-core Gram kernels.
//
// Lane L holds x[j] = G(row0 + L, col0 + j), j = 0..31; the block's elements
// with lag offset delta = j - L (-31..31) must be summed.  Adding every element
// to a lag counter in shared memory costs one shared atomic per element, which
// the atomic unit serves at about one element per SM clock -- slower than the
// MMAs of a short-K item.  Instead:
//   1. rotate each lane's 32 values left by its lane index (five conditional
//      power-of-two rotations, one select per value each): afterwards u[k] of
//      lane L is x[(k + L) mod 32], an element of lag offset k (when
//      k + L < 32) or k - 32 (otherwise);
//   2. for each k, two warp reductions (redux.sync) split at lane 32 - k give
//      the sums of lag offsets k and k - 32; lane k keeps both.
// So lane l ends with the block's sums for lag offsets l ("hi") and l - 32
// ("lo"; 0 for lane 0).  The exact integer values are summed in uint32: the
// caller guarantees a block's sum fits (every entry <= 2^24, 32 entries).
#pragma once
#include <cstdint>

namespace g2 {

__device__ __forceinline__ void rotate_by_lane(uint32_t (&u)[32], uint32_t lane) {
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const bool b = (lane >> s) & 1u;
    uint32_t t[32];
#pragma unroll
    for (int k = 0; k < 32; ++k) t[k] = b ? u[(k + (1 << s)) & 31] : u[k];
#pragma unroll
    for (int k = 0; k < 32; ++k) u[k] = t[k];
  }
}

// x: the lane's row of the block (consumed).  Returns the sums of lag
// offsets `lane` (hi) and `lane - 32` (lo) over the whole warp's block.
__device__ __forceinline__ void block_lag_sums(uint32_t (&x)[32], uint32_t lane, uint32_t& hi, uint32_t& lo) {
  rotate_by_lane(x, lane);
  hi = 0;
  lo = 0;
#pragma unroll
  for (int k = 0; k < 32; ++k) {
    const uint32_t h = lane < static_cast<uint32_t>(32 - k) ? x[k] : 0u;
    const uint32_t sh = __reduce_add_sync(0xffffffffu, h);
    const uint32_t sl = __reduce_add_sync(0xffffffffu, x[k] - h);
    if (lane == static_cast<uint32_t>(k)) {
      hi = sh;
      lo = sl;
    }
  }
}

}  // namespace g2
