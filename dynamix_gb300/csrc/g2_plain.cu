// G5: the plain direct numerator on CUDA cores -- the same-GPU comparator of
// the tensor-core Gram.
//
// It evaluates the same integer sums as correlator_multiQ_dense
// (densecorrelator.cl:6-56) -- N(tau) = sum_t sum_p I(t,p) I(t+tau,p) with
// 32-bit unsigned integer multiply-adds -- but register-tiled: a 256-thread
// block owns a 128 x 128 block of (t, t') pairs, each thread an 8 x 8 set of
// uint32 accumulators fed from shared memory, and the lag diagonals are summed
// in shared memory before the int64 atomics.  Operands are the packed 16-bit
// counts of G1 (raw integers), widened to 32 bits when they are staged.
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace plain {

constexpr int BM = G2_PLAIN_BM;  // 128
constexpr int BN = G2_PLAIN_BN;  // 128
constexpr int KT = 32;           // k per shared-memory tile
constexpr int LD = KT + 4;       // padded row (words)
constexpr int THREADS = 256;
constexpr int NDIAG = BM + BN - 1;  // 255
constexpr int TILE_WORDS = BM * LD;
constexpr int SMEM_BYTES = (2 * 2 * TILE_WORDS + 256) * 4;

struct JobsParam {
  const uint16_t* packed[G2_MAX_JOBS];
  int64_t cols[G2_MAX_JOBS];
  int64_t rows[G2_MAX_JOBS];
};

__device__ __forceinline__ bool item_ok(const g2_gram_item& w, int n_jobs, int64_t numer_len) {
  return w.job >= 0 && w.job < n_jobs && w.k_len > 0 && (w.k_len % KT) == 0 && (w.a_k0 % KT) == 0 &&
         (w.b_k0 % KT) == 0 && w.nframes > 0 && w.shift >= 0 && w.shift <= 32 && w.out_off >= 0 &&
         w.out_off + w.nframes <= numer_len && w.s_off < 0;
}

// Load rows [r0, r0+128) x cols [k, k+32) of a packed matrix: 512 chunks of
// 8 fp16, two per thread; rows beyond `rows` or columns beyond `cols` read 0.
__device__ __forceinline__ void load_tile(const uint16_t* __restrict__ base, int64_t cols, int64_t rows, int r0,
                                          int64_t k, uint4 (&reg)[2]) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = threadIdx.x + u * THREADS;
    const int r = e >> 2;
    const int c = (e & 3) * 8;
    const int64_t gr = static_cast<int64_t>(r0) + r;
    if (gr >= 0 && gr < rows && k + c + 8 <= cols)
      reg[u] = *reinterpret_cast<const uint4*>(base + gr * cols + k + c);
    else
      reg[u] = make_uint4(0, 0, 0, 0);
  }
}

// packed fp16 operands hold the raw integer counts (0..2048) as 16-bit values
__device__ __forceinline__ uint32_t h2u(uint32_t bits16) { return bits16; }

__device__ __forceinline__ void store_tile(uint32_t* __restrict__ s, const uint4 (&reg)[2]) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = threadIdx.x + u * THREADS;
    const int r = e >> 2;
    const int c = (e & 3) * 8;
    const uint32_t w[4] = {reg[u].x, reg[u].y, reg[u].z, reg[u].w};
    uint4 lo, hi;
    lo.x = h2u(w[0] & 0xffff);
    lo.y = h2u(w[0] >> 16);
    lo.z = h2u(w[1] & 0xffff);
    lo.w = h2u(w[1] >> 16);
    hi.x = h2u(w[2] & 0xffff);
    hi.y = h2u(w[2] >> 16);
    hi.z = h2u(w[3] & 0xffff);
    hi.w = h2u(w[3] >> 16);
    *reinterpret_cast<uint4*>(s + r * LD + c) = lo;
    *reinterpret_cast<uint4*>(s + r * LD + c + 4) = hi;
  }
}

__global__ void __launch_bounds__(THREADS, 2)
    plain_kernel(const __grid_constant__ JobsParam jobs, int n_jobs, const g2_gram_item* __restrict__ items,
                 int64_t n_items, unsigned long long* __restrict__ numer, int64_t numer_len,
                 int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  uint32_t* sA[2] = {sm, sm + TILE_WORDS};
  uint32_t* sB[2] = {sm + 2 * TILE_WORDS, sm + 3 * TILE_WORDS};
  uint32_t* dacc = sm + 4 * TILE_WORDS;  // 256 lag counters
  const int tx = threadIdx.x & 15;
  const int ty = threadIdx.x >> 4;

  for (int64_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const g2_gram_item w = items[it];
    if (!item_ok(w, n_jobs, numer_len)) {
      if (threadIdx.x == 0) atomicOr(err, G2_DEVERR_BOUNDS);
      continue;
    }
    const uint16_t* base = jobs.packed[w.job];
    const int64_t cols = jobs.cols[w.job];
    const int64_t rows = jobs.rows[w.job];
    dacc[threadIdx.x] = 0;

    uint32_t acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0;

    const int nkt = w.k_len / KT;
    uint4 ra[2], rb[2];
    load_tile(base, cols, rows, w.i0, w.a_k0, ra);
    load_tile(base, cols, rows, w.j0, w.b_k0, rb);
    store_tile(sA[0], ra);
    store_tile(sB[0], rb);
    __syncthreads();
    for (int kt = 0; kt < nkt; ++kt) {
      const int cur = kt & 1;
      if (kt + 1 < nkt) {
        load_tile(base, cols, rows, w.i0, w.a_k0 + static_cast<int64_t>(kt + 1) * KT, ra);
        load_tile(base, cols, rows, w.j0, w.b_k0 + static_cast<int64_t>(kt + 1) * KT, rb);
      }
      const uint32_t* a = sA[cur];
      const uint32_t* b = sB[cur];
#pragma unroll 1
      for (int k = 0; k < KT; k += 4) {
        uint4 av[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) av[i] = *reinterpret_cast<const uint4*>(a + (ty + 16 * i) * LD + k);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const uint4 bv = *reinterpret_cast<const uint4*>(b + (tx + 16 * j) * LD + k);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            acc[i][j] += av[i].x * bv.x;
            acc[i][j] += av[i].y * bv.y;
            acc[i][j] += av[i].z * bv.z;
            acc[i][j] += av[i].w * bv.w;
          }
        }
      }
      if (kt + 1 < nkt) {
        store_tile(sA[cur ^ 1], ra);
        store_tile(sB[cur ^ 1], rb);
      }
      __syncthreads();
    }
    // lag-diagonal sums: element (row ty+16i, col tx+16j), lag offset col - row
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j)
        if (acc[i][j]) atomicAdd(&dacc[(tx + 16 * j) - (ty + 16 * i) + (BM - 1)], acc[i][j]);
    __syncthreads();
    if (threadIdx.x < NDIAG) {
      const uint32_t s = dacc[threadIdx.x];
      const int tau = w.j0 - w.i0 + threadIdx.x - (BM - 1);
      if (s && tau >= 0 && tau < w.nframes)
        atomicAdd(&numer[w.out_off + tau], static_cast<unsigned long long>(s) << w.shift);
    }
    __syncthreads();
  }
}


// ---- u8 variant: four multiply-adds per __dp4a ------------------------------
// The same direct sums on the raw count bytes (the e4m3 pack's output is the
// u8 counts themselves): a 256-thread block owns a 128 x 128 block of (t, t')
// pairs, each thread an 8 x 8 set of uint32 accumulators, and every __dp4a
// adds four byte products.  An entry over k_len <= 65,536 columns is at most
// 65,536 * 255^2 < 2^32, so uint32 accumulators are exact for any u8 counts;
// the lag sums of a block are kept in uint64 shared counters.  The column of
// the packed matrix's row of ones (t' = nframes), when the item reaches it,
// gives the bin sums S(t) = G(t, nframes) as in the tensor-core path.
constexpr int KT8 = 64;             // bytes of k per shared-memory tile
constexpr int LD8 = KT8 / 4 + 4;    // padded row (words): conflict-free 16-byte loads
constexpr int TILE8_WORDS = BM * LD8;
constexpr int SMEM8_BYTES = 2 * 2 * TILE8_WORDS * 4 + 256 * 8;
constexpr int64_t MAX_K8 = 65536;

struct Jobs8Param {
  const uint8_t* packed[G2_MAX_JOBS];
  int64_t cols[G2_MAX_JOBS];
  int64_t rows[G2_MAX_JOBS];   // frames, + 1 with the row of ones
  int32_t ones[G2_MAX_JOBS];
};

__device__ __forceinline__ bool item8_ok(const g2_gram_item& w, const Jobs8Param& jp, int n_jobs,
                                         int64_t numer_len, int64_t sums_len) {
  return w.job >= 0 && w.job < n_jobs && w.k_len > 0 && w.k_len <= MAX_K8 && (w.k_len % KT8) == 0 &&
         (w.a_k0 % 16) == 0 && (w.b_k0 % 16) == 0 && w.nframes > 0 && w.shift >= 0 && w.shift <= 32 &&
         w.out_off >= 0 && w.out_off + w.nframes <= numer_len &&
         (w.s_off < 0 || (jp.ones[w.job] && w.shift == 0 && w.s_off + w.nframes <= sums_len));
}

// rows [r0, r0+128) x bytes [k, k+64): 512 chunks of 16 bytes, two per thread
__device__ __forceinline__ void load_tile8(const uint8_t* __restrict__ base, int64_t cols, int64_t rows, int r0,
                                           int64_t k, uint4 (&reg)[2]) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = threadIdx.x + u * THREADS;
    const int r = e >> 2;
    const int c = (e & 3) * 16;
    const int64_t gr = static_cast<int64_t>(r0) + r;
    if (gr >= 0 && gr < rows && k + c + 16 <= cols)
      reg[u] = *reinterpret_cast<const uint4*>(base + gr * cols + k + c);
    else
      reg[u] = make_uint4(0, 0, 0, 0);
  }
}

__device__ __forceinline__ void store_tile8(uint32_t* __restrict__ s, const uint4 (&reg)[2]) {
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int e = threadIdx.x + u * THREADS;
    *reinterpret_cast<uint4*>(s + (e >> 2) * LD8 + (e & 3) * 4) = reg[u];
  }
}

__global__ void __launch_bounds__(THREADS, 1)
    plain_dp4a_kernel(const __grid_constant__ Jobs8Param jobs, int n_jobs, const g2_gram_item* __restrict__ items,
                      int64_t n_items, unsigned long long* __restrict__ numer, int64_t numer_len,
                      unsigned long long* __restrict__ sums, int64_t sums_len, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm8[];
  uint32_t* sA[2] = {sm8, sm8 + TILE8_WORDS};
  uint32_t* sB[2] = {sm8 + 2 * TILE8_WORDS, sm8 + 3 * TILE8_WORDS};
  unsigned long long* dacc = reinterpret_cast<unsigned long long*>(sm8 + 4 * TILE8_WORDS);  // 256 lags
  const int tx = threadIdx.x & 15;
  const int ty = threadIdx.x >> 4;

  for (int64_t it = blockIdx.x; it < n_items; it += gridDim.x) {
    const g2_gram_item w = items[it];
    if (!item8_ok(w, jobs, n_jobs, numer_len, sums_len)) {
      if (threadIdx.x == 0) atomicOr(err, G2_DEVERR_BOUNDS);
      continue;
    }
    const uint8_t* base = jobs.packed[w.job];
    const int64_t cols = jobs.cols[w.job];
    const int64_t rows = jobs.rows[w.job];
    dacc[threadIdx.x] = 0ull;

    uint32_t acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0;

    const int nkt = w.k_len / KT8;
    uint4 ra[2], rb[2];
    load_tile8(base, cols, rows, w.i0, w.a_k0, ra);
    load_tile8(base, cols, rows, w.j0, w.b_k0, rb);
    store_tile8(sA[0], ra);
    store_tile8(sB[0], rb);
    __syncthreads();
    for (int kt = 0; kt < nkt; ++kt) {
      const int cur = kt & 1;
      if (kt + 1 < nkt) {
        load_tile8(base, cols, rows, w.i0, w.a_k0 + static_cast<int64_t>(kt + 1) * KT8, ra);
        load_tile8(base, cols, rows, w.j0, w.b_k0 + static_cast<int64_t>(kt + 1) * KT8, rb);
      }
      const uint32_t* a = sA[cur];
      const uint32_t* b = sB[cur];
#pragma unroll 1
      for (int k = 0; k < KT8 / 4; k += 4) {
        uint4 av[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) av[i] = *reinterpret_cast<const uint4*>(a + (ty + 16 * i) * LD8 + k);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const uint4 bv = *reinterpret_cast<const uint4*>(b + (tx + 16 * j) * LD8 + k);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            acc[i][j] = __dp4a(av[i].x, bv.x, acc[i][j]);
            acc[i][j] = __dp4a(av[i].y, bv.y, acc[i][j]);
            acc[i][j] = __dp4a(av[i].z, bv.z, acc[i][j]);
            acc[i][j] = __dp4a(av[i].w, bv.w, acc[i][j]);
          }
        }
      }
      if (kt + 1 < nkt) {
        store_tile8(sA[cur ^ 1], ra);
        store_tile8(sB[cur ^ 1], rb);
      }
      __syncthreads();
    }
    // lag-diagonal sums of the t' >= t elements with t, t' < nframes; the
    // column of the row of ones goes to the bin sums
    const int ones_c = w.s_off >= 0 ? w.nframes - w.j0 : -1;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int r = ty + 16 * i;
      if (w.i0 + r >= w.nframes) continue;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = tx + 16 * j;
        const uint32_t x = acc[i][j];
        if (!x) continue;
        if (c == ones_c)
          atomicAdd(&sums[w.s_off + w.i0 + r], static_cast<unsigned long long>(x));
        else if (w.j0 + c < w.nframes)
          atomicAdd(&dacc[c - r + (BM - 1)], static_cast<unsigned long long>(x));
      }
    }
    __syncthreads();
    if (threadIdx.x < NDIAG) {
      const unsigned long long s = dacc[threadIdx.x];
      const int tau = w.j0 - w.i0 + threadIdx.x - (BM - 1);
      if (s && tau >= 0 && tau < w.nframes) atomicAdd(&numer[w.out_off + tau], s << w.shift);
    }
    __syncthreads();
  }
}

}  // namespace plain
}  // namespace g2

extern "C" int g2_plain_direct(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                               uint64_t* numer_dev, int64_t numer_len, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !numer_dev || numer_len <= 0 || !err_dev)
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  plain::JobsParam jp;
  for (int j = 0; j < G2_MAX_JOBS; ++j) {
    jp.packed[j] = nullptr;
    jp.cols[j] = 0;
    jp.rows[j] = 0;
  }
  for (int j = 0; j < n_jobs; ++j) {
    const g2_job& jb = jobs[j];
    if (!jb.packed_dev || !aligned(jb.packed_dev, 16) || jb.nframes <= 0 || jb.nframes >= (1ll << 31) ||
        jb.packed_cols <= 0 || jb.packed_cols % G2_PAD != 0 || jb.elem_kind != G2_KIND_FP16 || jb.ones_row != 0)
      return G2_ERR_ARG;
    jp.packed[j] = reinterpret_cast<const uint16_t*>(jb.packed_dev);
    jp.cols[j] = jb.packed_cols;
    jp.rows[j] = jb.nframes;
  }
  if (n_items == 0) return G2_OK;
  if (cudaFuncSetAttribute(plain::plain_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, plain::SMEM_BYTES) !=
      cudaSuccess)
    return G2_ERR_CUDA;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  int64_t g = static_cast<int64_t>(sms) * 2;
  if (g > n_items) g = n_items;
  plain::plain_kernel<<<static_cast<unsigned>(g), plain::THREADS, plain::SMEM_BYTES, as_stream(stream)>>>(
      jp, n_jobs, items_dev, n_items, reinterpret_cast<unsigned long long*>(numer_dev), numer_len, err_dev);
  return launch_status();
}

extern "C" int g2_plain_dp4a(const g2_job* jobs, int32_t n_jobs, const g2_gram_item* items_dev, int64_t n_items,
                             uint64_t* numer_dev, int64_t numer_len, uint64_t* sums_dev, int64_t sums_len,
                             int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!jobs || n_jobs < 1 || n_jobs > G2_MAX_JOBS || n_items < 0 || !numer_dev || numer_len <= 0 || !err_dev ||
      sums_len < 0 || (sums_len > 0 && !sums_dev))
    return G2_ERR_ARG;
  if (n_items > 0 && !items_dev) return G2_ERR_ARG;
  plain::Jobs8Param jp;
  for (int j = 0; j < G2_MAX_JOBS; ++j) {
    jp.packed[j] = nullptr;
    jp.cols[j] = 0;
    jp.rows[j] = 0;
    jp.ones[j] = 0;
  }
  for (int j = 0; j < n_jobs; ++j) {
    const g2_job& jb = jobs[j];
    if (!jb.packed_dev || !aligned(jb.packed_dev, 16) || jb.nframes <= 0 || jb.nframes >= (1ll << 31) ||
        jb.packed_cols <= 0 || jb.packed_cols % G2_PAD != 0 || jb.elem_kind != G2_KIND_E4M3 ||
        (jb.ones_row != 0 && jb.ones_row != 1))
      return G2_ERR_ARG;
    jp.packed[j] = reinterpret_cast<const uint8_t*>(jb.packed_dev);
    jp.cols[j] = jb.packed_cols;
    jp.rows[j] = jb.nframes + jb.ones_row;
    jp.ones[j] = jb.ones_row;
  }
  if (n_items == 0) return G2_OK;
  if (cudaFuncSetAttribute(plain::plain_dp4a_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           plain::SMEM8_BYTES) != cudaSuccess)
    return G2_ERR_CUDA;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, plain::plain_dp4a_kernel, plain::THREADS,
                                                    plain::SMEM8_BYTES) != cudaSuccess ||
      per_sm < 1)
    return G2_ERR_CUDA;
  int64_t g = static_cast<int64_t>(sms) * per_sm;
  if (g > n_items) g = n_items;
  plain::plain_dp4a_kernel<<<static_cast<unsigned>(g), plain::THREADS, plain::SMEM8_BYTES, as_stream(stream)>>>(
      jp, n_jobs, items_dev, n_items, reinterpret_cast<unsigned long long*>(numer_dev), numer_len,
      reinterpret_cast<unsigned long long*>(sums_dev), sums_len, err_dev);
  return launch_status();
}
