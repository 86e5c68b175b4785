// Tensor-core rate probe: the dense MMA rate of this GPU for the two operand
// kinds the Gram uses, measured with this library's own tcgen05 code.
//
// Every CTA (one per SM) fills one A tile (128 rows x 128 B) and one B tile
// (256 rows x 128 B) of shared memory with count-like values (bytes 0..16 for
// e4m3; the 16-bit raw counts 0..16 for fp16, as the packed operands hold
// them), then one thread issues `iters` groups of four M128 N256 MMAs (K = 32
// e4m3 or 16 fp16 each, the Gram's stage) into one TMEM accumulator, back to
// back.  No global memory is touched in the loop, so the launch time measures
// the tensor pipe alone: MACs per launch = grid * iters * 4 * 128 * 256 * K.
// The Gram's roofline is stated against this rate (there is no kind::i8 on
// sm_103a, and no library GEMM runs kind::f8f6f4 on raw integer counts).
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace peak {

constexpr int BM = 128;
constexpr int BN = 256;
constexpr int ROW_BYTES = 128;
constexpr int A_BYTES = BM * ROW_BYTES;
constexpr int B_BYTES = BN * ROW_BYTES;
constexpr int THREADS = 128;
constexpr int SMEM_BYTES = 1024 + A_BYTES + B_BYTES + 64;
constexpr uint32_t IDESC = idesc_f32acc(BM, BN);

template <int KIND>
__global__ void __launch_bounds__(THREADS, 1) tc_rate_kernel(int64_t iters, int32_t* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + A_BYTES;
  uint64_t* done = reinterpret_cast<uint64_t*>(smem + A_BYTES + B_BYTES);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(done + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5;

  // count-like operand values: e4m3 bytes 0..16, or fp16 words 0..16
  uint32_t* w32 = reinterpret_cast<uint32_t*>(smem);
  for (int i = threadIdx.x; i < (A_BYTES + B_BYTES) / 4; i += THREADS) {
    const uint32_t h = (static_cast<uint32_t>(i) * 2654435761u) ^ blockIdx.x;
    if (KIND == G2_KIND_E4M3)
      w32[i] = (h & 0x0F0F0F0Fu) + ((h >> 4) & 0x01010101u);
    else
      w32[i] = (h & 0x000F000Fu) + ((h >> 4) & 0x00010001u);
  }
  if (threadIdx.x == 0) {
    mbar_init(done, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  // make the generic-proxy stores visible to the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (warp == 0) tmem_alloc(tmem_slot, BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    const uint32_t a0 = smem_addr(sA), b0 = smem_addr(sB);
    for (int64_t it = 0; it < iters; ++it) {
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        if (KIND == G2_KIND_E4M3)
          tc_mma_f8f6f4(tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), IDESC,
                        (it | kk) != 0 ? 1u : 0u);
        else
          tc_mma_f16(tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), IDESC,
                     (it | kk) != 0 ? 1u : 0u);
      }
    }
    tc_commit(done);
    // bounded: records G2_DEVERR_TIMEOUT instead of hanging
    mbar_wait(done, 0, abort_flag, err);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, BN);
  }
}

}  // namespace peak
}  // namespace g2

extern "C" int g2_tc_rate_probe(int32_t kind, int64_t iters, int32_t grid, int32_t* err_dev, void* stream) {
  using namespace g2;
  if ((kind != G2_KIND_FP16 && kind != G2_KIND_E4M3) || iters <= 0 || iters > (1ll << 31) || grid < 0 ||
      !err_dev)
    return G2_ERR_ARG;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int g = grid > 0 ? grid : sms;
  if (kind == G2_KIND_E4M3) {
    if (cudaFuncSetAttribute(peak::tc_rate_kernel<G2_KIND_E4M3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             peak::SMEM_BYTES) != cudaSuccess)
      return G2_ERR_CUDA;
    peak::tc_rate_kernel<G2_KIND_E4M3><<<g, peak::THREADS, peak::SMEM_BYTES, as_stream(stream)>>>(iters, err_dev);
  } else {
    if (cudaFuncSetAttribute(peak::tc_rate_kernel<G2_KIND_FP16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             peak::SMEM_BYTES) != cudaSuccess)
      return G2_ERR_CUDA;
    peak::tc_rate_kernel<G2_KIND_FP16><<<g, peak::THREADS, peak::SMEM_BYTES, as_stream(stream)>>>(iters, err_dev);
  }
  return launch_status();
}
