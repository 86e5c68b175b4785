// G2: tensor-core Gram of each q-bin's (frames x pixels) matrix with the
// lag-diagonal sums fused into the epilogue.
//
// For one item, the CTA computes the 128 x 256 block G(t, t') = sum_k A(t,k) B(t',k)
// (t = i0 + r, t' = j0 + c) with tcgen05.mma into TMEM -- kind::f16 on 16-bit
// counts <= 2048 or kind::f8f6f4 on 8-bit counts <= 16 (half the bytes and
// twice the MMA rate), chosen per job -- then adds
// every element with t' >= t to the lag tau = t' - t:
//     N(tau) += 2^shift * sum_{c - r = tau - (j0 - i0)} G(r, c).
// The Gram never reaches HBM.  The packed operands are the raw integer counts:
// read as e4m3, the bytes 0..16 are exactly count * 2^-9 (subnormals and the
// first binades); read as fp16, the 16-bit values 0..2048 are exactly
// count * 2^-24.  Products are exact in fp32 and the caller splits K so that
// every partial sum is an integer below 2^24 times that power of two; the
// epilogue rescales (exact), converts each element to uint32, sums the lag
// diagonals of each 32 x 32 block in registers and then in uint32 shared
// counters (<= 128 * 2^24 < 2^32), which are added to the int64 numerator.
//
// Roles (192 threads, one CTA per SM, persistent over a static item schedule):
//   warp 0 lane 0  TMA producer: A (128 x 64) and B (256 x 64) fp16 tiles per
//                  stage, 4-stage ring, 128-byte swizzle
//   warp 1 lane 0  MMA issuer: 4 x (M128 N256 K16) per stage into one of two
//                  TMEM accumulators (2 x 256 columns)
//   warps 2..5     epilogue: tcgen05.ld 32 columns at a time, lag sums by
//                  lane rotation and warp reductions, int64 atomics to the
//                  numerator
// Replaces dense.py:54,61-64 (numpy sgemm + diagonal loop), cuda.py:67-116
// (cuBLAS sgemm + extract_upper_diags) and densecorrelator.cl:6-56.
#include <cstring>
#include <mutex>
#include "g2_epilogue.cuh"
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace tc {

constexpr int BM = G2_TC_BM;      // 128 rows of A per item (TMEM lanes)
constexpr int BN = G2_TC_BN;      // 256 rows of B per item (TMEM columns)
constexpr int ROW_BYTES = 128;   // bytes per operand row per stage (64 fp16 or 128 e4m3)
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * ROW_BYTES;
constexpr int B_BYTES = BN * ROW_BYTES;
constexpr int STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int NDIAG = BM + BN - 1;  // lags covered by one item
constexpr int NDIAG_PAD = 384;
constexpr int TMEM_COLS = 2 * BN;
constexpr int NUM_THREADS = 192;
constexpr int EPI_THREADS = 128;
constexpr uint32_t IDESC = idesc_f32acc(BM, BN);  // same bits for fp16 and e4m3 operands

constexpr int SMEM_BAR_OFF = STAGES * STAGE_BYTES;
constexpr int SMEM_BYTES = 1024 /*alignment slack*/ + SMEM_BAR_OFF + 256 + 2 * NDIAG_PAD * 4;
// deviation mode: per TMEM buffer the lag centres, sums of d, sums of d^2 and
// zero-denominator counts (4 x NDIAG_PAD words)
constexpr int STD_WORDS = 4 * NDIAG_PAD;
constexpr int SMEM_BYTES_STD = 1024 + SMEM_BAR_OFF + 256 + 2 * STD_WORDS * 4;

// Outputs of the deviation mode (calc_std of dense.py:58-66): for every pair
// t' >= t of one bin, r = P G(t,t') / (S(t) S(t')) and d = r - centre(tau);
// the lag sums of d and d^2 (float per block, double in memory) and the count
// of pairs with S(t) S(t') = 0.
// The two-time mode (the TTCF of event_y.py:148-157) writes the same r for
// every pair t' > t of one bin into a row-major matrix (row stride ld), and
// its mirror (t', t) when `mirror` is set.
struct StdOut {
  const long long* S;      // bin sums, indexed by item.s_off + t
  const float* centre;     // per lag, indexed by item.out_off + tau
  double* sum_d;           // indexed by item.out_off + tau
  double* sum_d2;
  unsigned int* zeros;
  float* ttcf;             // two-time mode: [n][ld]
  int64_t ld;
  int64_t n;
  int mirror;
};

// Epilogue modes of the Gram kernel.
constexpr int MODE_NUMER = 0;  // lag sums of G (the numerator)
constexpr int MODE_STD = 1;    // deviation of the per-pair ratio (calc_std)
constexpr int MODE_TTCF = 2;   // per-pair ratio written as the two-time matrix
constexpr int MODE_MATRIX = 3; // 2^shift G(t,t') for t' >= t written (or added) to a matrix

struct MapsParam {
  CUtensorMap a[G2_MAX_JOBS];
  CUtensorMap b[G2_MAX_JOBS];
  int32_t kind[G2_MAX_JOBS];  // G2_KIND_FP16 or G2_KIND_E4M3
  int32_t ones[G2_MAX_JOBS];  // packed matrix has the row of ones at row nframes
};

// packed elements per 128-byte stage row
__device__ __forceinline__ int stage_elems(int kind) { return kind == G2_KIND_E4M3 ? 128 : 64; }

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

// Every role applies the same test, so a malformed item is skipped by all of
// them consistently (the epilogue records G2_DEVERR_BOUNDS).
// In the deviation mode ``shift`` carries the bin's pixel count and ``s_off``
// the offset of its sums.
template <int MODE>
__device__ __forceinline__ bool item_ok(const g2_gram_item& w, const MapsParam& maps, int n_jobs,
                                        int64_t numer_len, int64_t sums_len, int64_t max_frames) {
  constexpr bool STD = MODE == MODE_STD || MODE == MODE_TTCF;
  if ((MODE == MODE_TTCF || MODE == MODE_MATRIX) && w.nframes > max_frames) return false;
  if (w.job < 0 || w.job >= n_jobs) return false;
  const int bk = stage_elems(maps.kind[w.job]);
  const bool shape = w.k_len > 0 && (w.k_len % bk) == 0 && (w.a_k0 % bk) == 0 && (w.b_k0 % bk) == 0 &&
                     w.nframes > 0 && w.out_off >= 0 && w.out_off + w.nframes <= numer_len;
  if (MODE == MODE_MATRIX) return shape && w.shift >= 0 && w.shift <= 30;
  if (STD) return shape && w.shift > 0 && w.s_off >= 0 && w.s_off + w.nframes <= sums_len;
  return shape && w.shift >= 0 && w.shift <= 32 &&
         (w.s_off < 0 || (maps.ones[w.job] && w.shift == 0 && w.s_off + w.nframes <= sums_len));
}

template <int MODE>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    gram_tc_kernel(const __grid_constant__ MapsParam maps, int n_jobs, const g2_gram_item* __restrict__ items,
                   int64_t n_items, unsigned long long* __restrict__ numer, int64_t numer_len,
                   unsigned long long* __restrict__ sums, int64_t sums_len, int32_t* __restrict__ err,
                   const StdOut so) {
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

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accf[b], 1);
      mbar_init(&acce[b], EPI_THREADS);
    }
    mbar_init(drain, 1);
    *abort_flag = 0;
    fence_mbar_init();
  }
  constexpr bool STD = MODE != MODE_NUMER;
  for (int i = threadIdx.x; i < (STD ? 2 * STD_WORDS : 2 * NDIAG_PAD); i += NUM_THREADS) diag[i] = 0;
  if (warp == 1) tmem_alloc(tmem_slot, TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t issued = 0;
      bool ok = true;
      for (int64_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        const g2_gram_item w = items[it];
        if (w.job == G2_ITEM_EMPTY) continue;
        if (!item_ok<MODE>(w, maps, n_jobs, numer_len, sums_len, so.n)) continue;
        const CUtensorMap* ma = &maps.a[w.job];
        const CUtensorMap* mb = &maps.b[w.job];
        const int bk = stage_elems(maps.kind[w.job]);
        const int nk = w.k_len / bk;
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err)) {
            ok = false;
            break;
          }
          mbar_arrive_expect_tx(&full[stage], STAGE_BYTES);
          tma_load_2d(sA + stage * A_BYTES, ma, &full[stage], w.a_k0 + kb * bk, w.i0);
          tma_load_2d(sB + stage * B_BYTES, mb, &full[stage], w.b_k0 + kb * bk, w.j0);
          ++issued;
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
      // Make sure no TMA write into this CTA's shared memory is still in
      // flight when the CTA exits (returns at once on the normal path).
      const int64_t last = issued < STAGES ? issued : STAGES;
      for (int64_t k = 1; k <= last; ++k) {
        const int64_t idx = issued - k;
        mbar_wait_drain(&full[idx % STAGES], static_cast<uint32_t>((idx / STAGES) & 1), 200000000ull);
      }
    }
    __syncwarp();
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int64_t local = 0;
      bool ok = true;
      for (int64_t it = blockIdx.x; it < n_items && ok; it += gridDim.x) {
        const g2_gram_item w = items[it];
        if (w.job == G2_ITEM_EMPTY) continue;
        if (!item_ok<MODE>(w, maps, n_jobs, numer_len, sums_len, so.n)) continue;
        const bool fp8 = maps.kind[w.job] == G2_KIND_E4M3;
        const int buf = static_cast<int>(local & 1);
        const uint32_t ap = static_cast<uint32_t>((local >> 1) & 1);
        if (!mbar_wait(&acce[buf], ap ^ 1, abort_flag, err)) break;
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + static_cast<uint32_t>(buf * BN);
        const int nk = w.k_len / stage_elems(maps.kind[w.job]);
        for (int kb = 0; kb < nk; ++kb) {
          if (!mbar_wait(&full[stage], phase, abort_flag, err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a0 = smem_addr(sA + stage * A_BYTES);
          const uint32_t b0 = smem_addr(sB + stage * B_BYTES);
          // four MMAs of 32 bytes of K each (K = 16 fp16 or 32 e4m3)
          if (fp8) {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              tc_mma_f8f6f4(d_tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), IDESC,
                            (kb | kk) != 0 ? 1u : 0u);
          } else {
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              tc_mma_f16(d_tmem, smem_desc_sw128(a0 + kk * 32), smem_desc_sw128(b0 + kk * 32), IDESC,
                         (kb | kk) != 0 ? 1u : 0u);
          }
          tc_commit(&empty[stage]);
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
        if (ok) tc_commit(&accf[buf]);
        ++local;
      }
      // All MMAs issued by this thread complete before TMEM is released.
      tc_commit(drain);
      mbar_wait_drain(drain, 0, 200000000ull);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int q = warp & 3;  // TMEM sub-partition this warp may access
    const int row = q * 32 + lane;
    const int etid = threadIdx.x - 64;
    int64_t local = 0;
    for (int64_t it = blockIdx.x; it < n_items; it += gridDim.x, ++local) {
      const g2_gram_item w = items[it];
      if (w.job == G2_ITEM_EMPTY) {
        --local;
        continue;
      }
      if (!item_ok<MODE>(w, maps, n_jobs, numer_len, sums_len, so.n)) {
        if (etid == 0) atomicOr(err, G2_DEVERR_BOUNDS);
        --local;
        continue;
      }
      const int buf = static_cast<int>(local & 1);
      const uint32_t ap = static_cast<uint32_t>((local >> 1) & 1);
      uint32_t* dacc = diag + (local & 1) * NDIAG_PAD;
      const bool ok = mbar_wait(&accf[buf], ap, abort_flag, err);
      if (named_bar_any(1, EPI_THREADS, !ok)) break;
      tc_fence_after();
      // packed counts are raw integers read as e4m3 (count * 2^-9) or fp16
      // (count * 2^-24): each accumulator holds sum * 2^-18 or sum * 2^-48
      const float unscale = maps.kind[w.job] == G2_KIND_E4M3 ? 262144.0f : 281474976710656.0f;
      const uint32_t tbase = tmem_base + (static_cast<uint32_t>(q * 32) << 16) + static_cast<uint32_t>(buf * BN);
      // frames >= nframes (TMA zero fill, or the row of ones) never enter the
      // lag sums; the column of the row of ones, when this block holds it,
      // goes to the bin sums instead
      const bool row_live = w.i0 + row < w.nframes;
      const int col_end = min(BN, w.nframes - w.j0);                // columns < col_end are frames
      const int lag0 = w.j0 - w.i0 - (BM - 1);
      if (MODE == MODE_MATRIX) {
        // ---------------------------------------- Gram matrix mode epilogue
        // this item's plane combination of the bin, weighted by 2^shift, for
        // every pair t' >= t; `mirror` set: added to what earlier launches wrote
        const float wgt = unscale * static_cast<float>(1u << w.shift);
        const int64_t t = static_cast<int64_t>(w.i0) + row;
#pragma unroll 1
        for (int cc = 0; cc < BN / 32; ++cc) {
          uint32_t v[32];
          __syncwarp();
          tmem_ld_32x32b_x32(tbase + static_cast<uint32_t>(cc * 32), v);
          tmem_wait_ld();
          if (!row_live) continue;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int c = cc * 32 + j;
            const int64_t t2 = static_cast<int64_t>(w.j0) + c;
            if (c >= col_end || t2 < t) continue;  // t' >= T, or below the diagonal
            float* o = so.ttcf + t * so.ld + t2;
            const float g = __uint_as_float(v[j]) * wgt;
            *o = so.mirror ? *o + g : g;
          }
        }
        tc_fence_before();
        mbar_arrive(&acce[buf]);
        continue;
      }
      if (MODE == MODE_TTCF) {
        // ---------------------------------------- two-time mode epilogue
        const float P = static_cast<float>(w.shift);
        const int64_t t = static_cast<int64_t>(w.i0) + row;
        const float St = row_live ? static_cast<float>(so.S[w.s_off + t]) : 0.0f;
#pragma unroll 1
        for (int cc = 0; cc < BN / 32; ++cc) {
          uint32_t v[32];
          __syncwarp();
          tmem_ld_32x32b_x32(tbase + static_cast<uint32_t>(cc * 32), v);
          tmem_wait_ld();
          if (!row_live) continue;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int c = cc * 32 + j;
            const int64_t t2 = static_cast<int64_t>(w.j0) + c;
            if (c >= col_end || t2 <= t) continue;  // t' >= T, or not above the diagonal
            const float den = St * static_cast<float>(so.S[w.s_off + t2]);
            const float r = P * (__uint_as_float(v[j]) * unscale) / den;  // 0/0 -> NaN as in the reference
            so.ttcf[t * so.ld + t2] = r;
            if (so.mirror) so.ttcf[t2 * so.ld + t] = r;
          }
        }
        tc_fence_before();
        mbar_arrive(&acce[buf]);
        continue;
      }
      if (MODE == MODE_STD) {
        // ---------------------------------------- deviation mode epilogue
        float* cen = reinterpret_cast<float*>(diag) + (local & 1) * STD_WORDS;
        float* sd = cen + NDIAG_PAD;
        float* sd2 = sd + NDIAG_PAD;
        unsigned int* zc = reinterpret_cast<unsigned int*>(sd2 + NDIAG_PAD);
        for (int d = etid; d < NDIAG; d += EPI_THREADS) {
          const int tau = lag0 + d;
          const float c = (tau >= 0 && tau < w.nframes) ? so.centre[w.out_off + tau] : 0.0f;
          cen[d] = isfinite(c) ? c : 0.0f;
        }
        named_bar_sync(1, EPI_THREADS);
        const float P = static_cast<float>(w.shift);
        const float St = row_live ? static_cast<float>(so.S[w.s_off + w.i0 + row]) : 0.0f;
#pragma unroll 1
        for (int cc = 0; cc < BN / 32; ++cc) {
          uint32_t v[32];
          __syncwarp();
          tmem_ld_32x32b_x32(tbase + static_cast<uint32_t>(cc * 32), v);
          tmem_wait_ld();
          if (!row_live) continue;
          const int dbase = cc * 32 - row + (BM - 1);
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (cc * 32 + j >= col_end || dbase + j < (BM - 1) - (w.j0 - w.i0)) continue;  // t' >= T or t' < t
            const float den = St * static_cast<float>(so.S[w.s_off + w.j0 + cc * 32 + j]);
            if (den == 0.0f) {
              atomicAdd(&zc[dbase + j], 1u);
            } else {
              const float r = P * (__uint_as_float(v[j]) * unscale) / den;
              const float dv = r - cen[dbase + j];
              atomicAdd(&sd[dbase + j], dv);
              atomicAdd(&sd2[dbase + j], dv * dv);
            }
          }
        }
        tc_fence_before();
        mbar_arrive(&acce[buf]);
        named_bar_sync(1, EPI_THREADS);
        for (int d = etid; d < NDIAG; d += EPI_THREADS) {
          const int tau = lag0 + d;
          if (tau >= 0 && tau < w.nframes) {
            if (sd[d] != 0.0f) atomicAdd(&so.sum_d[w.out_off + tau], static_cast<double>(sd[d]));
            if (sd2[d] != 0.0f) atomicAdd(&so.sum_d2[w.out_off + tau], static_cast<double>(sd2[d]));
            if (zc[d]) atomicAdd(&so.zeros[w.out_off + tau], zc[d]);
          }
          sd[d] = 0.0f;
          sd2[d] = 0.0f;
          zc[d] = 0u;
        }
        continue;
      }
      const int ones_col = w.s_off >= 0 ? w.nframes - w.j0 : -1;  // -1 or >= BN: not in this block
      // rows past the frames (the row of ones among them) contribute nothing;
      // columns past the frames are TMA zero fill, except the row of ones,
      // whose column goes to the bin sums.  Lag sums of each 32 x 32 block in
      // registers (g2_epilogue.cuh), one shared add per lane and lag group.
      const float us = row_live ? unscale : 0.0f;
      const int dwarp = (BM - 1) - q * 32 + lane;  // lag index of offset `lane` in chunk 0
      uint32_t carry = 0;
#pragma unroll 1
      for (int cc = 0; cc < BN / 32; ++cc) {
        uint32_t v[32];
        __syncwarp();  // tcgen05.ld is warp-collective: reconverge after the previous chunk
        tmem_ld_32x32b_x32(tbase + static_cast<uint32_t>(cc * 32), v);
        tmem_wait_ld();
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = __float2uint_rn(__uint_as_float(v[j]) * us);
        const int jx = ones_col - cc * 32;
        if (jx >= 0 && jx < 32) {  // warp-uniform
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (j == jx) {
              if (v[j]) atomicAdd(&sums[w.s_off + w.i0 + row], static_cast<unsigned long long>(v[j]));
              v[j] = 0;
            }
        }
        uint32_t hi, lo;
        block_lag_sums(v, static_cast<uint32_t>(lane), hi, lo);
        const uint32_t val = carry + lo;  // lag group cc - 1 is complete
        const int d = (cc - 1) * 32 + dwarp;
        if (val && d >= 0) atomicAdd(&dacc[d], val);
        carry = hi;
      }
      if (carry) atomicAdd(&dacc[(BN / 32 - 1) * 32 + dwarp], carry);
      tc_fence_before();
      mbar_arrive(&acce[buf]);
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

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, TMEM_COLS);
  }
}

}  // namespace tc
}  // namespace g2

namespace {
template <int MODE>
int launch_gram(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len, int32_t* err_dev,
                int32_t grid, void* stream, const g2::tc::StdOut& so) {
  using namespace g2;
  for (int j = 0; j < n_jobs; ++j) {
    const g2_job& jb = jobs[j];
    if (!jb.packed_dev || !aligned(jb.packed_dev, 16) || jb.nframes <= 0 || jb.nframes >= (1ll << 31) ||
        jb.packed_cols <= 0 || jb.packed_cols % G2_PAD != 0 || jb.packed_cols >= (1ll << 31) ||
        (jb.elem_kind != G2_KIND_FP16 && jb.elem_kind != G2_KIND_E4M3) || (jb.ones_row != 0 && jb.ones_row != 1))
      return G2_ERR_ARG;
  }
  if (n_items == 0) return G2_OK;
  static tc::MapsParam maps;  // large; filled under the lock below
  static std::mutex* mu = new std::mutex;
  std::lock_guard<std::mutex> lk(*mu);
  std::memset(&maps, 0, sizeof(maps));
  for (int j = 0; j < n_jobs; ++j) {
    const int eb = jobs[j].elem_kind == G2_KIND_E4M3 ? 1 : 2;
    const uint32_t box_cols = tc::ROW_BYTES / eb;
    const uint64_t rows = static_cast<uint64_t>(jobs[j].nframes) + (jobs[j].ones_row ? 1 : 0);
    int st = encode_tmap_2d(&maps.a[j], jobs[j].packed_dev, eb, jobs[j].packed_cols, rows, box_cols, tc::BM);
    if (st != G2_OK) return st;
    st = encode_tmap_2d(&maps.b[j], jobs[j].packed_dev, eb, jobs[j].packed_cols, rows, box_cols, tc::BN);
    if (st != G2_OK) return st;
    maps.kind[j] = jobs[j].elem_kind;
    maps.ones[j] = jobs[j].ones_row;
  }
  const int smem = MODE != tc::MODE_NUMER ? tc::SMEM_BYTES_STD : tc::SMEM_BYTES;
  if (cudaFuncSetAttribute(tc::gram_tc_kernel<MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return G2_ERR_CUDA;
  int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  int64_t g = grid > 0 ? grid : sms;
  if (g > n_items) g = n_items;
  tc::gram_tc_kernel<MODE><<<static_cast<unsigned>(g), tc::NUM_THREADS, smem, as_stream(stream)>>>(
      maps, n_jobs, items_dev, n_items, reinterpret_cast<unsigned long long*>(numer_dev), numer_len,
      reinterpret_cast<unsigned long long*>(sums_dev), sums_len, err_dev, so);
  return launch_status();
}
}  // namespace

extern "C" int g2_gram_tc(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                          uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
                          int32_t* err_dev, int32_t grid, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !numer_dev || numer_len <= 0 || !err_dev ||
      sums_len < 0 || (sums_len > 0 && !sums_dev))
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  const tc::StdOut none = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0, 0, 0};
  return launch_gram<tc::MODE_NUMER>(jobs, n_jobs, items_dev, n_items, numer_dev, numer_len, sums_dev, sums_len, err_dev,
                            grid, stream, none);
}

extern "C" int g2_gram_std(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                           const int64_t* sums_dev, int64_t sums_len, const float* centre_dev, double* sum_d_dev,
                           double* sum_d2_dev, uint32_t* zeros_dev, int64_t out_len, int32_t* err_dev,
                           int32_t grid, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !sums_dev || sums_len <= 0 || !centre_dev ||
      !sum_d_dev || !sum_d2_dev || !zeros_dev || out_len <= 0 || !err_dev)
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  const tc::StdOut so = {reinterpret_cast<const long long*>(sums_dev), centre_dev, sum_d_dev, sum_d2_dev,
                         zeros_dev, nullptr, 0, 0, 0};
  // out_len bounds out_off + tau, sums_len bounds s_off + t; numer and sums
  // are not written in this mode
  return launch_gram<tc::MODE_STD>(jobs, n_jobs, items_dev, n_items, reinterpret_cast<uint64_t*>(sum_d_dev), out_len,
                           reinterpret_cast<uint64_t*>(const_cast<int64_t*>(sums_dev)), sums_len, err_dev, grid,
                           stream, so);
}

namespace g2 {
namespace tc {
// Below the diagonal when the matrix is not mirrored: 0 where S(t) S(t') != 0,
// NaN where it is 0 (the reference's 0 * P / (S S) there).
__global__ void __launch_bounds__(256)
    ttcf_lower_kernel(float* __restrict__ out, int64_t n, int64_t ld, const long long* __restrict__ S) {
  for (int64_t t = blockIdx.x; t < n; t += gridDim.x) {
    const long long st = S[t];
    for (int64_t t2 = threadIdx.x; t2 < t; t2 += blockDim.x)
      out[t * ld + t2] = (st != 0 && S[t2] != 0) ? 0.0f : __int_as_float(0x7fc00000);
  }
}

// The diagonal: every element but the last is the mean of the positive
// elements of the first upper diagonal (NaN when there are none); the last is
// 0, or NaN when S(T - 1) = 0.
__global__ void __launch_bounds__(1024)
    ttcf_diag_kernel(float* __restrict__ out, int64_t n, int64_t ld, const long long* __restrict__ S) {
  __shared__ double s_sum[32];
  __shared__ unsigned long long s_cnt[32];
  double sum = 0.0;
  unsigned long long cnt = 0;
  for (int64_t j = threadIdx.x; j + 1 < n; j += blockDim.x) {
    const float x = out[j * ld + j + 1];
    if (x > 0.0f) {
      sum += x;
      ++cnt;
    }
  }
  for (int o = 16; o; o >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) {
    s_sum[warp] = sum;
    s_cnt[warp] = cnt;
  }
  __syncthreads();
  if (warp == 0) {
    sum = lane < (blockDim.x >> 5) ? s_sum[lane] : 0.0;
    cnt = lane < (blockDim.x >> 5) ? s_cnt[lane] : 0ull;
    for (int o = 16; o; o >>= 1) {
      sum += __shfl_xor_sync(0xffffffffu, sum, o);
      cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    }
    if (lane == 0) {
      s_sum[0] = sum;
      s_cnt[0] = cnt;
    }
  }
  __syncthreads();
  const float mean = s_cnt[0] ? static_cast<float>(s_sum[0] / static_cast<double>(s_cnt[0]))
                              : __int_as_float(0x7fc00000);
  for (int64_t j = threadIdx.x; j + 1 < n; j += blockDim.x) out[j * ld + j] = mean;
  if (threadIdx.x == 0) out[(n - 1) * ld + (n - 1)] = S[n - 1] != 0 ? 0.0f : __int_as_float(0x7fc00000);
}
}  // namespace tc
}  // namespace g2

extern "C" int g2_gram_ttcf(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                            const int64_t* sums_dev, int64_t sums_len, float* ttcf_dev, int64_t nframes, int64_t ld,
                            int32_t mirror, int32_t* err_dev, int32_t grid, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !sums_dev || sums_len <= 0 || !ttcf_dev ||
      nframes <= 0 || ld < nframes || !err_dev)
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  const tc::StdOut so = {reinterpret_cast<const long long*>(sums_dev), nullptr, nullptr, nullptr, nullptr,
                         ttcf_dev, ld, nframes, mirror ? 1 : 0};
  // items address S through s_off (bounded by sums_len) and may not have more
  // frames than the matrix; numer is not written in this mode
  return launch_gram<tc::MODE_TTCF>(jobs, n_jobs, items_dev, n_items, nullptr, sums_len,
                                    reinterpret_cast<uint64_t*>(const_cast<int64_t*>(sums_dev)), sums_len, err_dev,
                                    grid, stream, so);
}

extern "C" int g2_gram_matrix(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                              float* matrix_dev, int64_t nframes, int64_t ld, int32_t accumulate, int32_t* err_dev,
                              int32_t grid, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !matrix_dev || nframes <= 0 || ld < nframes ||
      !err_dev)
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  const tc::StdOut so = {nullptr, nullptr, nullptr, nullptr, nullptr, matrix_dev, ld, nframes, accumulate ? 1 : 0};
  // items may not have more frames than the matrix (out_off + nframes bounded by nframes);
  // numer and sums are not written in this mode
  return launch_gram<tc::MODE_MATRIX>(jobs, n_jobs, items_dev, n_items, nullptr, nframes, nullptr, 0, err_dev, grid,
                                      stream, so);
}

extern "C" int g2_ttcf_finish(float* ttcf_dev, int64_t nframes, int64_t ld, const int64_t* bin_sums_dev,
                              int32_t mirror, void* stream) {
  using namespace g2;
  if (!ttcf_dev || !bin_sums_dev || nframes <= 0 || ld < nframes) return G2_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  const long long* S = reinterpret_cast<const long long*>(bin_sums_dev);
  if (!mirror) {
    const int64_t blocks = nframes < 65536 ? nframes : 65536;
    tc::ttcf_lower_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(ttcf_dev, nframes, ld, S);
  }
  tc::ttcf_diag_kernel<<<1, 1024, 0, st>>>(ttcf_dev, nframes, ld, S);
  return launch_status();
}
