// G2 on CTA pairs: the tensor-core Gram of each q-bin's (frames x pixels)
// matrix on 256 x 256 blocks, with the lag-diagonal sums fused into the
// epilogue, one tcgen05 cta_group::2 MMA per K step shared by two SMs.
//
// A cluster of two CTAs owns one item at a time: the block G(t, t') for
// t in [i0, i0 + 256), t' in [j0, j0 + n) with n = min(256, the frames (and
// row of ones) left from j0, rounded up to 32).  Each CTA loads its own half
// of A (rows i0 + 128 r ...) and its own half of B (rows j0 + r n/2 ...) into
// its own shared memory -- 32 KB per stage per CTA instead of the 48 KB a
// single-CTA 128 x 256 block needs -- and the leader CTA (rank 0) issues the
// pair MMA M256 N n, which reads both CTAs' halves; CTA r's TMEM receives
// rows i0 + 128 r ... of the block.  So each SM streams a third less from L2
// per MMA cycle, and the ring holds six stages.  The arithmetic and the
// exactness argument are those of the single-CTA kernel (g2_gram_tc.cu):
// e4m3 bytes 0..16 = count * 2^-9 or fp16 words 0..2048 = count * 2^-24,
// fp32 sums kept below 2^24 by the caller's K split, int64 atomics to the
// numerator.  The epilogue sums each 32 x 32 block's lag diagonals in
// registers (g2_epilogue.cuh), then adds one value per lane and lag group to
// uint32 shared counters.
//
// Roles per CTA (192 threads): warp 0 lane 0 TMA producer (both CTAs), warp 1
// lane 0 MMA issuer (leader only; warp 1 of both CTAs allocates TMEM), warps
// 2..5 epilogue (both CTAs, each on its own TMEM rows).
// Barriers: full[s] of the leader collects both CTAs' TMA bytes of stage s;
// empty[s] of each CTA and accf[b] of each CTA are signalled by the leader's
// commits (multicast); acce[b] of the leader collects one arrival per
// epilogue warp of both CTAs.  Every wait is bounded (G2_DEVERR_TIMEOUT).
// Replaces the same reference code as g2_gram_tc: dense.py:54,61-64,
// cuda.py:67-116, densecorrelator.cl:6-56.
#include <cstring>
#include <mutex>
#include "g2_epilogue.cuh"
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace pair {

constexpr int BM = 256;                 // rows of A per item (128 per CTA)
constexpr int BN = 256;                 // largest MMA N (columns per item)
constexpr int HALF = 128;               // rows of A and of B each CTA loads per stage
constexpr int ROW_BYTES = 128;          // 64 fp16 or 128 e4m3 per row per stage
constexpr int STAGES = 6;
constexpr int A_BYTES = HALF * ROW_BYTES;
constexpr int B_BYTES = HALF * ROW_BYTES;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;  // per CTA
constexpr int NDIAG = HALF + BN - 1;            // lags of one CTA's 128 x 256 part
constexpr int NDIAG_PAD = 384;
constexpr int TMEM_COLS = 2 * BN;
constexpr int NUM_THREADS = 192;
constexpr int EPI_THREADS = 128;
constexpr int EPI_WARPS = EPI_THREADS / 32;
constexpr int SMEM_BAR_OFF = STAGES * STAGE_BYTES;
constexpr int SMEM_BYTES = 1024 /*alignment slack*/ + SMEM_BAR_OFF + 256 + 2 * NDIAG_PAD * 4;
static_assert(SMEM_BYTES <= 227 * 1024, "shared memory of one CTA");

struct MapsParam {
  CUtensorMap map[G2_MAX_JOBS];  // box: one stage row (128 B) x 128 rows, 128-byte swizzle
  int32_t kind[G2_MAX_JOBS];
  int32_t ones[G2_MAX_JOBS];
};

__device__ __forceinline__ int stage_elems(int kind) { return kind == G2_KIND_E4M3 ? 128 : 64; }

// Columns of the item's MMA: the frames (and the row of ones) left from j0,
// rounded up to a multiple of 32, at most 256.
__device__ __forceinline__ int item_n(const g2_gram_item& w, const MapsParam& maps) {
  const int live = w.nframes + (w.s_off >= 0 && maps.ones[w.job] ? 1 : 0) - w.j0;
  const int n = (live + 31) & ~31;
  return n < 32 ? 32 : (n > BN ? BN : n);
}

__device__ __forceinline__ bool item_ok(const g2_gram_item& w, const MapsParam& maps, int n_jobs,
                                        int64_t numer_len, int64_t sums_len) {
  if (w.job < 0 || w.job >= n_jobs) return false;
  const int bk = stage_elems(maps.kind[w.job]);
  return w.k_len > 0 && (w.k_len % bk) == 0 && (w.a_k0 % bk) == 0 && (w.b_k0 % bk) == 0 && w.nframes > 0 &&
         w.i0 >= 0 && w.j0 >= 0 && w.j0 < w.nframes + 1 && w.out_off >= 0 && w.out_off + w.nframes <= numer_len &&
         w.shift >= 0 && w.shift <= 32 &&
         (w.s_off < 0 || (maps.ones[w.job] && w.shift == 0 && w.s_off + w.nframes <= sums_len));
}

__device__ __forceinline__ bool named_bar_any(uint32_t id, uint32_t n, bool v) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred p, q;\n\t"
      "setp.ne.u32 q, %3, 0;\n\t"
      "bar.red.or.pred p, %1, %2, q;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(r)
      : "r"(id), "r"(n), "r"(static_cast<uint32_t>(v))
      : "memory");
  return r != 0;
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(NUM_THREADS, 1)
    gram_pair_kernel(const __grid_constant__ MapsParam maps, int n_jobs, const g2_gram_item* __restrict__ items,
                     int64_t n_items, unsigned long long* __restrict__ numer, int64_t numer_len,
                     unsigned long long* __restrict__ sums, int64_t sums_len, int32_t* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* sA = smem;
  uint8_t* sB = smem + STAGES * A_BYTES;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + SMEM_BAR_OFF);
  uint64_t* empty = full + STAGES;
  uint64_t* accf = empty + STAGES;
  uint64_t* acce = accf + 2;
  uint64_t* drain = acce + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  uint32_t* diag = reinterpret_cast<uint32_t*>(smem + SMEM_BAR_OFF + 256);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint32_t rank = cluster_ctarank();
  const int64_t cluster = blockIdx.x >> 1;
  const int64_t n_clusters = gridDim.x >> 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);   // the leader's arrive.expect_tx; both CTAs' bytes
      mbar_init(&empty[s], 1);  // the leader's commit (multicast)
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], 2 * EPI_WARPS);  // one per epilogue warp of both CTAs (leader's copy)
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < 2 * NDIAG_PAD; i += NUM_THREADS) diag[i] = 0;
  // both CTAs have initialised their barriers (and are running) before any
  // signal crosses between them
  cluster_sync_all();
  if (warp == 1) tmem_alloc_pair(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer (both CTAs)
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t issued = 0;
      bool ok = true;
      for (int64_t it = cluster; it < n_items && ok; it += n_clusters) {
        const g2_gram_item w = items[it];
        if (w.job == G2_ITEM_EMPTY) continue;
        if (!item_ok(w, maps, n_jobs, numer_len, sums_len)) continue;
        const CUtensorMap* m = &maps.map[w.job];
        const int bk = stage_elems(maps.kind[w.job]);
        const int nk = w.k_len / bk;
        const int n = item_n(w, maps);
        const int32_t arow = w.i0 + static_cast<int32_t>(rank) * HALF;
        const int32_t brow = w.j0 + static_cast<int32_t>(rank) * (n / 2);
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait_cluster(&empty[stage], phase ^ 1, abort_flag, err)) {
            ok = false;
            break;
          }
          if (rank == 0) mbar_arrive_expect_tx(&full[stage], 2 * STAGE_BYTES);
          const uint32_t fb = mapa_shared(smem_addr(&full[stage]), 0);
          tma_load_2d_pair(sA + stage * A_BYTES, m, fb, w.a_k0 + kb * bk, arow);
          tma_load_2d_pair(sB + stage * B_BYTES, m, fb, w.b_k0 + kb * bk, brow);
          ++issued;
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // The leader sees its stages complete; both CTAs' last stages are
      // consumed by MMAs that the leader drains before the final cluster
      // barrier, so no TMA write is in flight when the CTAs exit.
      if (rank == 0) {
        const int64_t last = issued < STAGES ? issued : STAGES;
        for (int64_t k = 1; k <= last; ++k) {
          const int64_t idx = issued - k;
          mbar_wait_drain(&full[idx % STAGES], static_cast<uint32_t>((idx / STAGES) & 1), 200000000ull);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer (leader)
    if (lane == 0 && rank == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t local = 0;
      bool ok = true;
      for (int64_t it = cluster; it < n_items && ok; it += n_clusters) {
        const g2_gram_item w = items[it];
        if (w.job == G2_ITEM_EMPTY) continue;
        if (!item_ok(w, maps, n_jobs, numer_len, sums_len)) continue;
        const bool fp8 = maps.kind[w.job] == G2_KIND_E4M3;
        const int n = item_n(w, maps);
        const uint32_t idesc = idesc_f32acc(BM, static_cast<uint32_t>(n));
        const int buf = static_cast<int>(local & 1);
        const uint32_t ap = static_cast<uint32_t>((local >> 1) & 1);
        if (!mbar_wait_cluster(&acce[buf], ap ^ 1, abort_flag, err)) break;
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + static_cast<uint32_t>(buf * BN);
        const int nk = w.k_len / stage_elems(maps.kind[w.job]);
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait_cluster(&full[stage], phase, abort_flag, err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_addr(sA + stage * A_BYTES);
          const uint32_t b0 = smem_addr(sB + stage * B_BYTES);
          if (fp8) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              tc_mma_pair_f8f6f4(d_tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), idesc,
                                 (kb | kk) != 0 ? 1u : 0u);
          } else {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              tc_mma_pair_f16(d_tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), idesc,
                              (kb | kk) != 0 ? 1u : 0u);
          }
          tc_commit_pair_mc(&empty[stage], 0x3);
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (ok) tc_commit_pair_mc(&accf[buf], 0x3);
        ++local;
      }
      // every MMA issued here completes before TMEM is released
      tc_commit_pair(drain);
      mbar_wait_drain(drain, 0, 200000000ull);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue (both CTAs)
    const int q = warp & 3;  // TMEM sub-partition this warp may access
    const int row = q * 32 + lane;
    const int etid = threadIdx.x - 64;
    int64_t local = 0;
    for (int64_t it = cluster; it < n_items; it += n_clusters, ++local) {
      const g2_gram_item w = items[it];
      if (w.job == G2_ITEM_EMPTY) {
        --local;
        continue;
      }
      if (!item_ok(w, maps, n_jobs, numer_len, sums_len)) {
        if (etid == 0 && rank == 0) atomicOr(err, G2_DEVERR_BOUNDS);
        --local;
        continue;
      }
      const int buf = static_cast<int>(local & 1);
      const uint32_t ap = static_cast<uint32_t>((local >> 1) & 1);
      uint32_t* dacc = diag + (local & 1) * NDIAG_PAD;
      const bool ok = mbar_wait_cluster(&accf[buf], ap, abort_flag, err);
      if (named_bar_any(1, EPI_THREADS, !ok)) break;
      tc_fence_after();
      const float unscale = maps.kind[w.job] == G2_KIND_E4M3 ? 262144.0f : 281474976710656.0f;
      const uint32_t tbase = tmem_base + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(buf * BN);
      const int i0 = w.i0 + static_cast<int>(rank) * HALF;  // first frame of this CTA's rows
      const bool row_live = i0 + row < w.nframes;
      const int n = item_n(w, maps);
      const int lag0 = w.j0 - i0 - (HALF - 1);
      const int ones_col = w.s_off >= 0 ? w.nframes - w.j0 : -1;  // -1 or >= n: not in this block
      // rows past the frames (the row of ones among them) contribute nothing;
      // columns past the frames are TMA zero fill, except the row of ones,
      // whose column goes to the bin sums
      const float us = row_live ? unscale : 0.0f;
      const int dwarp = (HALF - 1) - q * 32 + lane;  // lag index of offset `lane` in chunk 0
      uint32_t carry = 0;
#pragma unroll 1
      for (int cc = 0; cc < n / 32; ++cc) {
        uint32_t v[32];
        __syncwarp();  // tcgen05.ld is warp-collective
        tmem_ld_32x32b_x32(tbase + static_cast<uint32_t>(cc * 32), v);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = __float2uint_rn(__uint_as_float(v[j]) * us);
        const int jx = ones_col - cc * 32;
        if (jx >= 0 && jx < 32) {  // warp-uniform
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (j == jx) {
              if (v[j]) atomicAdd(&sums[w.s_off + i0 + row], static_cast<unsigned long long>(v[j]));
              v[j] = 0;
            }
        }
        uint32_t hi, lo;
        block_lag_sums(v, static_cast<uint32_t>(lane), hi, lo);
        // lag group cc - 1 is complete: this chunk's lo and the previous chunk's hi
        const uint32_t val = carry + lo;
        const int d = (cc - 1) * 32 + dwarp;
        if (val && d >= 0) atomicAdd(&dacc[d], val);
        carry = hi;
      }
      if (carry) atomicAdd(&dacc[(n / 32 - 1) * 32 + dwarp], carry);
      // this warp's TMEM reads are done: release the buffer to the leader's MMA
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive_cluster(mapa_shared(smem_addr(&acce[buf]), 0));
      named_bar_sync(1, EPI_THREADS);
      for (int d = etid; d < NDIAG; d += EPI_THREADS) {
        const uint32_t s = dacc[d];
        if (s) {
          const int tau = lag0 + d;
          if (tau >= 0 && tau < w.nframes)
            atomicAdd(&numer[w.out_off + tau], static_cast<unsigned long long>(s) << w.shift);
          dacc[d] = 0;
        }
      }
    }
  }

  // After a timed-out wait a TMA of this CTA may still be landing: give it
  // time before the pair leaves (the normal path has drained everything).
  if (*abort_flag) {
    const uint64_t t0 = global_timer_ns();
    while (global_timer_ns() - t0 < 100000ull) {
    }
  }
  tc_fence_before();
  __syncthreads();
  // neither CTA exits (or frees TMEM) while the other may still signal it
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc_pair(tmem_base, TMEM_COLS);
  }
}


// ---- wide items: 256 x 512 blocks ------------------------------------------
// The same pair MMA twice per K step, on two 256-column halves of B that share
// the stage's A rows: each CTA streams 16 KB of A and 2 x 16 KB of B per 1024
// MMA cycles (48 B per cycle instead of the 64 of a 256 x 256 item), and the
// 4-stage ring looks 4096 MMA cycles ahead.  The accumulator takes all 512
// TMEM columns, so an item's epilogue is not overlapped with the next item's
// MMAs: these items suit long K (the autotuner chooses per workload).  A half
// that lies wholly below the diagonal (j0 + 256 <= i0) is skipped, and each
// half's width is the frames (and row of ones) it holds, rounded up to 32.
constexpr int W_BN = 512;
constexpr int W_STAGES = 4;
constexpr int W_STAGE_BYTES = A_BYTES + 2 * B_BYTES;  // per CTA
constexpr int W_NDIAG = HALF + W_BN - 1;
constexpr int W_NDIAG_PAD = 640;
constexpr int W_SMEM_BAR_OFF = W_STAGES * W_STAGE_BYTES;
constexpr int W_SMEM_BYTES = 1024 + W_SMEM_BAR_OFF + 256 + 2 * W_NDIAG_PAD * 4;
static_assert(W_SMEM_BYTES <= 227 * 1024, "shared memory of one CTA");

// Widths of the two halves of a wide item (0: the half is skipped).
__device__ __forceinline__ void wide_halves(const g2_gram_item& w, const MapsParam& maps, int& n0, int& n1) {
  const int live = w.nframes + (w.s_off >= 0 && maps.ones[w.job] ? 1 : 0) - w.j0;
  const int r = (live + 31) & ~31;
  n0 = (w.j0 + HALF * 2 <= w.i0) ? 0 : (r > BN ? BN : (r < 32 ? 32 : r));
  const int r1 = r - BN;
  n1 = r1 <= 0 ? 0 : (r1 > BN ? BN : r1);
}

__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(NUM_THREADS, 1)
    gram_wide_kernel(const __grid_constant__ MapsParam maps, int n_jobs, const g2_gram_item* __restrict__ items,
                     int64_t n_items, unsigned long long* __restrict__ numer, int64_t numer_len,
                     unsigned long long* __restrict__ sums, int64_t sums_len, int32_t* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + W_SMEM_BAR_OFF);
  uint64_t* empty = full + W_STAGES;
  uint64_t* accf = empty + W_STAGES;
  uint64_t* acce = accf + 1;
  uint64_t* drain = acce + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  uint32_t* diag = reinterpret_cast<uint32_t*>(smem + W_SMEM_BAR_OFF + 256);

  const int warp = threadIdx.x >> 5;
  const int lane = threadIdx.x & 31;
  const uint32_t rank = cluster_ctarank();
  const int64_t cluster = blockIdx.x >> 1;
  const int64_t n_clusters = gridDim.x >> 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < W_STAGES; ++s) {
      mbar_init(&full[s], 1);   // the leader's arrive.expect_tx; both CTAs' bytes
      mbar_init(&empty[s], 1);  // the leader's commit (multicast)
    }
    mbar_init(accf, 1);
    mbar_init(acce, 2 * EPI_WARPS);  // one per epilogue warp of both CTAs (leader's copy)
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  for (int i = threadIdx.x; i < 2 * W_NDIAG_PAD; i += NUM_THREADS) diag[i] = 0;
  cluster_sync_all();
  if (warp == 1) tmem_alloc_pair(tmem_slot, 2 * BN);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer (both CTAs)
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t issued = 0;
      bool ok = true;
      for (int64_t it = cluster; it < n_items && ok; it += n_clusters) {
        const g2_gram_item w = items[it];
        if (w.job == G2_ITEM_EMPTY) continue;
        if (!item_ok(w, maps, n_jobs, numer_len, sums_len)) continue;
        const CUtensorMap* m = &maps.map[w.job];
        const int bk = stage_elems(maps.kind[w.job]);
        const int nk = w.k_len / bk;
        int n0, n1;
        wide_halves(w, maps, n0, n1);
        const uint32_t bytes = 2u * (A_BYTES + (n0 ? B_BYTES : 0) + (n1 ? B_BYTES : 0));
        const int32_t arow = w.i0 + static_cast<int32_t>(rank) * HALF;
        const int32_t brow0 = w.j0 + static_cast<int32_t>(rank) * (n0 / 2);
        const int32_t brow1 = w.j0 + BN + static_cast<int32_t>(rank) * (n1 / 2);
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait_cluster(&empty[stage], phase ^ 1, abort_flag, err)) {
            ok = false;
            break;
          }
          if (rank == 0) mbar_arrive_expect_tx(&full[stage], bytes);
          const uint32_t fb = mapa_shared(smem_addr(&full[stage]), 0);
          uint8_t* st = smem + stage * W_STAGE_BYTES;
          const int32_t kc = w.a_k0 + kb * bk;
          tma_load_2d_pair(st, m, fb, kc, arow);
          if (n0) tma_load_2d_pair(st + A_BYTES, m, fb, w.b_k0 + kb * bk, brow0);
          if (n1) tma_load_2d_pair(st + A_BYTES + B_BYTES, m, fb, w.b_k0 + kb * bk, brow1);
          ++issued;
          if (++stage == W_STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      if (rank == 0) {
        const int64_t last = issued < W_STAGES ? issued : W_STAGES;
        for (int64_t k = 1; k <= last; ++k) {
          const int64_t idx = issued - k;
          mbar_wait_drain(&full[idx % W_STAGES], static_cast<uint32_t>((idx / W_STAGES) & 1), 200000000ull);
        }
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer (leader)
    if (lane == 0 && rank == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t local = 0;
      bool ok = true;
      for (int64_t it = cluster; it < n_items && ok; it += n_clusters) {
        const g2_gram_item w = items[it];
        if (w.job == G2_ITEM_EMPTY) continue;
        if (!item_ok(w, maps, n_jobs, numer_len, sums_len)) continue;
        const bool fp8 = maps.kind[w.job] == G2_KIND_E4M3;
        int n0, n1;
        wide_halves(w, maps, n0, n1);
        const uint32_t id0 = idesc_f32acc(BM, static_cast<uint32_t>(n0 ? n0 : 32));
        const uint32_t id1 = idesc_f32acc(BM, static_cast<uint32_t>(n1 ? n1 : 32));
        if (!mbar_wait_cluster(acce, static_cast<uint32_t>(local & 1) ^ 1u, abort_flag, err)) break;
        tc_fence_after();
        const int nk = w.k_len / stage_elems(maps.kind[w.job]);
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait_cluster(&full[stage], phase, abort_flag, err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_addr(smem + stage * W_STAGE_BYTES);
          const uint32_t b0 = a0 + A_BYTES, b1 = a0 + A_BYTES + B_BYTES;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint32_t acc = (kb | kk) != 0 ? 1u : 0u;
            const uint64_t ad = smem_desc_sw128(a0 + kk * 32);
            if (fp8) {
              if (n0) tc_mma_pair_f8f6f4(tmem_base, ad, smem_desc_sw128(b0 + kk * 32), id0, acc);
              if (n1) tc_mma_pair_f8f6f4(tmem_base + BN, ad, smem_desc_sw128(b1 + kk * 32), id1, acc);
            } else {
              if (n0) tc_mma_pair_f16(tmem_base, ad, smem_desc_sw128(b0 + kk * 32), id0, acc);
              if (n1) tc_mma_pair_f16(tmem_base + BN, ad, smem_desc_sw128(b1 + kk * 32), id1, acc);
            }
          }
          tc_commit_pair_mc(&empty[stage], 0x3);
          if (++stage == W_STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (ok) tc_commit_pair_mc(accf, 0x3);
        ++local;
      }
      tc_commit_pair(drain);
      mbar_wait_drain(drain, 0, 200000000ull);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue (both CTAs)
    const int q = warp & 3;
    const int row = q * 32 + lane;
    const int etid = threadIdx.x - 64;
    int64_t local = 0;
    for (int64_t it = cluster; it < n_items; it += n_clusters, ++local) {
      const g2_gram_item w = items[it];
      if (w.job == G2_ITEM_EMPTY) {
        --local;
        continue;
      }
      if (!item_ok(w, maps, n_jobs, numer_len, sums_len)) {
        if (etid == 0 && rank == 0) atomicOr(err, G2_DEVERR_BOUNDS);
        --local;
        continue;
      }
      uint32_t* dacc = diag + (local & 1) * W_NDIAG_PAD;
      const bool ok = mbar_wait_cluster(accf, static_cast<uint32_t>(local & 1), abort_flag, err);
      if (named_bar_any(1, EPI_THREADS, !ok)) break;
      tc_fence_after();
      const float unscale = maps.kind[w.job] == G2_KIND_E4M3 ? 262144.0f : 281474976710656.0f;
      const uint32_t tbase = tmem_base + (static_cast<uint32_t>(q * 32) << 16);
      const int i0 = w.i0 + static_cast<int>(rank) * HALF;
      const bool row_live = i0 + row < w.nframes;
      int n0, n1;
      wide_halves(w, maps, n0, n1);
      // the item's columns are chunks [c_first, c_last) of 32: the left half's
      // n0 (none when skipped), then the right half's n1 (n0 < 256 => n1 = 0)
      const int c_first = n0 ? 0 : BN / 32;
      const int c_last = n1 ? (BN + n1) / 32 : n0 / 32;
      const int lag0 = w.j0 - i0 - (HALF - 1);
      const int ones_col = w.s_off >= 0 ? w.nframes - w.j0 : -1;
      const float us = row_live ? unscale : 0.0f;
      const int dwarp = (HALF - 1) - q * 32 + lane;
      uint32_t carry = 0;
      if (c_first >= c_last) {  // no columns (only for items that are not upper-triangle blocks)
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive_cluster(mapa_shared(smem_addr(acce), 0));
      }
#pragma unroll 1
      for (int cc = c_first; cc < c_last; ++cc) {
        uint32_t v[32];
        __syncwarp();
        tmem_ld_32x32b_x32(tbase + static_cast<uint32_t>(cc * 32), v);
        tmem_wait_ld();
        if (cc == c_last - 1) {
          // the last TMEM read of the item: release the accumulator now
          tc_fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive_cluster(mapa_shared(smem_addr(acce), 0));
        }
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = __float2uint_rn(__uint_as_float(v[j]) * us);
        const int jx = ones_col - cc * 32;
        if (jx >= 0 && jx < 32) {  // warp-uniform
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (j == jx) {
              if (v[j]) atomicAdd(&sums[w.s_off + i0 + row], static_cast<unsigned long long>(v[j]));
              v[j] = 0;
            }
        }
        uint32_t hi, lo;
        block_lag_sums(v, static_cast<uint32_t>(lane), hi, lo);
        const uint32_t val = carry + lo;
        const int d = (cc - 1) * 32 + dwarp;
        if (val && d >= 0) atomicAdd(&dacc[d], val);
        carry = hi;
      }
      if (carry) atomicAdd(&dacc[(c_last - 1) * 32 + dwarp], carry);  // carry != 0 only if the loop ran
      named_bar_sync(1, EPI_THREADS);
      for (int d = etid; d < W_NDIAG; d += EPI_THREADS) {
        const uint32_t s = dacc[d];
        if (s) {
          const int tau = lag0 + d;
          if (tau >= 0 && tau < w.nframes)
            atomicAdd(&numer[w.out_off + tau], static_cast<unsigned long long>(s) << w.shift);
          dacc[d] = 0;
        }
      }
    }
  }

  if (*abort_flag) {
    const uint64_t t0 = global_timer_ns();
    while (global_timer_ns() - t0 < 100000ull) {
    }
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync_all();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc_pair(tmem_base, 2 * BN);
  }
}

}  // namespace pair
}  // namespace g2

namespace {
// CTA pairs of `kernel` (one CTA per SM, `smem` bytes) that can be resident at once.
int max_clusters(const void* kernel, int smem, int* out) {
  using namespace g2;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess)
    return G2_ERR_CUDA;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(sms & ~1), 1, 1);
  cfg.blockDim = dim3(pair::NUM_THREADS, 1, 1);
  cfg.dynamicSmemBytes = smem;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, kernel, &cfg) != cudaSuccess || n < 1) return G2_ERR_CUDA;
  *out = n;
  return G2_OK;
}

int pair_max_clusters(int* out) {
  return max_clusters(reinterpret_cast<const void*>(g2::pair::gram_pair_kernel), g2::pair::SMEM_BYTES, out);
}

int wide_max_clusters(int* out) {
  return max_clusters(reinterpret_cast<const void*>(g2::pair::gram_wide_kernel), g2::pair::W_SMEM_BYTES, out);
}

// Checks the jobs and fills the tensor maps (box: 128 rows of one stage row).
int pair_maps(const g2_job* jobs, int32_t n_jobs, g2::pair::MapsParam* maps) {
  using namespace g2;
  for (int j = 0; j < n_jobs; ++j) {
    const g2_job& jb = jobs[j];
    if (!jb.packed_dev || !aligned(jb.packed_dev, 16) || jb.nframes <= 0 || jb.nframes >= (1ll << 31) ||
        jb.packed_cols <= 0 || jb.packed_cols % G2_PAD != 0 || jb.packed_cols >= (1ll << 31) ||
        (jb.elem_kind != G2_KIND_FP16 && jb.elem_kind != G2_KIND_E4M3) || (jb.ones_row != 0 && jb.ones_row != 1))
      return G2_ERR_ARG;
  }
  std::memset(maps, 0, sizeof(*maps));
  for (int j = 0; j < n_jobs; ++j) {
    const int eb = jobs[j].elem_kind == G2_KIND_E4M3 ? 1 : 2;
    const uint64_t rows = static_cast<uint64_t>(jobs[j].nframes) + (jobs[j].ones_row ? 1 : 0);
    const int st = encode_tmap_2d(&maps->map[j], jobs[j].packed_dev, eb, jobs[j].packed_cols, rows,
                                  pair::ROW_BYTES / eb, pair::HALF);
    if (st != G2_OK) return st;
    maps->kind[j] = jobs[j].elem_kind;
    maps->ones[j] = jobs[j].ones_row;
  }
  return G2_OK;
}
}  // namespace

extern "C" int g2_gram_workers(int32_t pair, int32_t* workers) {
  using namespace g2;
  if (!workers || pair < 0 || pair > 2) return G2_ERR_ARG;
  if (pair) {
    int n = 0;
    const int st = pair == 2 ? wide_max_clusters(&n) : pair_max_clusters(&n);
    if (st != G2_OK) return st;
    *workers = n;
    return G2_OK;
  }
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  *workers = sms;
  return G2_OK;
}

namespace {
int launch_pair(bool wide, const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len, int32_t* err_dev,
                int32_t grid, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !numer_dev || numer_len <= 0 || !err_dev ||
      sums_len < 0 || (sums_len > 0 && !sums_dev))
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  static pair::MapsParam maps;  // large; filled under the lock below
  static std::mutex* mu = new std::mutex;
  std::lock_guard<std::mutex> lk(*mu);
  int st = pair_maps(jobs, n_jobs, &maps);
  if (st != G2_OK) return st;
  if (n_items == 0) return G2_OK;
  int max_cl = 0;
  st = wide ? wide_max_clusters(&max_cl) : pair_max_clusters(&max_cl);
  if (st != G2_OK) return st;
  int64_t clusters = grid > 0 ? (grid + 1) / 2 : max_cl;
  if (clusters > max_cl) clusters = max_cl;
  if (clusters > n_items) clusters = n_items;
  const unsigned g = static_cast<unsigned>(2 * clusters);
  auto* nm = reinterpret_cast<unsigned long long*>(numer_dev);
  auto* sm = reinterpret_cast<unsigned long long*>(sums_dev);
  if (wide)
    pair::gram_wide_kernel<<<g, pair::NUM_THREADS, pair::W_SMEM_BYTES, as_stream(stream)>>>(
        maps, n_jobs, items_dev, n_items, nm, numer_len, sm, sums_len, err_dev);
  else
    pair::gram_pair_kernel<<<g, pair::NUM_THREADS, pair::SMEM_BYTES, as_stream(stream)>>>(
        maps, n_jobs, items_dev, n_items, nm, numer_len, sm, sums_len, err_dev);
  return launch_status();
}
}  // namespace

extern "C" int g2_gram_tc_pair(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                               uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
                               int32_t* err_dev, int32_t grid, void* stream) {
  return launch_pair(false, jobs, n_jobs, items_dev, n_items, numer_dev, numer_len, sums_dev, sums_len, err_dev, grid,
                     stream);
}

extern "C" int g2_gram_tc_wide(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                               uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
                               int32_t* err_dev, int32_t grid, void* stream) {
  return launch_pair(true, jobs, n_jobs, items_dev, n_items, numer_dev, numer_len, sums_dev, sums_len, err_dev, grid,
                     stream);
}
