// G7: per-frame CSR -> per-pixel event lists, so that the sparse correlator
// reuses the event pair-sum kernel (G6).
//
// CSR layout of dynamix's SparseCorrelator (intensity.py:70-77,
// correlator.cl:110-217): frame t owns elements [offsets[t], offsets[t+1]);
// indptr[t * (H+1) + r] .. indptr[t * (H+1) + r + 1] are the elements of row r
// relative to offsets[t]; indices[] is the column inside the row, data[] the
// count.  The transposition is a counting sort by pixel:
//   1. count   : events per pixel (global atomics)
//   2. scan    : exclusive prefix sum of the counts -> event offsets
//   3. scatter : each element takes the next slot of its pixel (atomic
//                cursor) and writes (t, v); the order inside a pixel is free
//                because G6 uses |t_j - t_i|.
// A warp walks one row of one frame (rows hold a handful of elements), a
// block one frame.
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace csr {

constexpr int THREADS = 256;
constexpr int WARPS = THREADS / 32;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 8;                        // elements per thread per scan block
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename Tv, typename Ti, bool SCATTER>
__global__ void __launch_bounds__(THREADS)
    walk_kernel(const Tv* __restrict__ data, const Ti* __restrict__ indices, const Ti* __restrict__ indptr,
                const Ti* __restrict__ offsets, int64_t n_elem, int32_t T, int32_t H, int32_t W,
                uint32_t* __restrict__ count_or_cursor, const uint32_t* __restrict__ ev_off,
                int32_t* __restrict__ ev_times, Tv* __restrict__ ev_data, int32_t* __restrict__ err) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  bool bad = false;
  for (int64_t t = blockIdx.x; t < T; t += gridDim.x) {
    const int64_t base = static_cast<int64_t>(offsets[t]);
    const int64_t fend = static_cast<int64_t>(offsets[t + 1]);
    const Ti* ip = indptr + t * static_cast<int64_t>(H + 1);
    for (int r = warp; r < H; r += WARPS) {
      const int64_t s = base + static_cast<int64_t>(ip[r]);
      const int64_t e = base + static_cast<int64_t>(ip[r + 1]);
      if (s < base || e < s || e > fend || e > n_elem) {
        bad = true;
        continue;
      }
      for (int64_t k = s + lane; k < e; k += 32) {
        const int64_t col = static_cast<int64_t>(indices[k]);
        if (col < 0 || col >= W) {
          bad = true;
          continue;
        }
        const int64_t pix = static_cast<int64_t>(r) * W + col;
        if (!SCATTER) {
          atomicAdd(&count_or_cursor[pix], 1u);
        } else {
          const uint32_t slot = ev_off[pix] + atomicAdd(&count_or_cursor[pix], 1u);
          if (slot < ev_off[pix + 1]) {
            ev_times[slot] = static_cast<int32_t>(t);
            ev_data[slot] = data[k];
          } else {
            bad = true;
          }
        }
      }
    }
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Exclusive scan of n uint32 into uint32 (the total must stay below 2^32):
// per tile sums, a single-block scan of the tile sums, then the tile scans.
__global__ void __launch_bounds__(SCAN_THREADS) tile_sums_kernel(const uint32_t* __restrict__ in, int64_t n,
                                                                 uint32_t* __restrict__ tile_sum) {
  __shared__ uint32_t ws[SCAN_THREADS / 32];
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * SCAN_TILE;
  uint32_t s = 0;
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    const int64_t k = t0 + static_cast<int64_t>(i) * SCAN_THREADS + threadIdx.x;
    if (k < n) s += in[k];
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    uint32_t v = threadIdx.x < SCAN_THREADS / 32 ? ws[threadIdx.x] : 0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = v;
  }
}

// In-place exclusive scan of up to SCAN_TILE values by one block.
__device__ void block_exclusive_scan(uint32_t (&v)[SCAN_ITEMS], uint32_t carry_in, uint32_t* ws) {
  // thread-local inclusive
  uint32_t tot = 0;
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    const uint32_t x = v[i];
    v[i] = tot;
    tot += x;
  }
  // warp scan of thread totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t inc = tot;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) ws[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = lane < SCAN_THREADS / 32 ? ws[lane] : 0;
    uint32_t wi = w;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += y;
    }
    if (lane < SCAN_THREADS / 32) ws[lane] = wi - w;  // exclusive warp offsets
  }
  __syncthreads();
  const uint32_t off = carry_in + ws[warp] + (inc - tot);
  for (int i = 0; i < SCAN_ITEMS; ++i) v[i] += off;
  __syncthreads();
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_sums_kernel(uint32_t* __restrict__ tile_sum, int64_t n_tiles,
                                                                      uint32_t* __restrict__ total) {
  __shared__ uint32_t ws[SCAN_THREADS / 32];
  uint32_t carry = 0;
  for (int64_t t0 = 0; t0 < n_tiles; t0 += SCAN_TILE) {
    uint32_t v[SCAN_ITEMS];
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const int64_t k = t0 + static_cast<int64_t>(threadIdx.x) * SCAN_ITEMS + i;
      v[i] = k < n_tiles ? tile_sum[k] : 0;
    }
    uint32_t chunk_total = 0;
    {
      uint32_t s = 0;
      for (int i = 0; i < SCAN_ITEMS; ++i) s += v[i];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      __shared__ uint32_t red[SCAN_THREADS / 32];
      if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
      __syncthreads();
      for (int w = 0; w < SCAN_THREADS / 32; ++w) chunk_total += red[w];
      __syncthreads();
    }
    block_exclusive_scan(v, carry, ws);
    for (int i = 0; i < SCAN_ITEMS; ++i) {
      const int64_t k = t0 + static_cast<int64_t>(threadIdx.x) * SCAN_ITEMS + i;
      if (k < n_tiles) tile_sum[k] = v[i];
    }
    carry += chunk_total;
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tiles_kernel(const uint32_t* __restrict__ in, int64_t n,
                                                                  const uint32_t* __restrict__ tile_off,
                                                                  uint32_t* __restrict__ out) {
  __shared__ uint32_t ws[SCAN_THREADS / 32];
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * SCAN_TILE;
  uint32_t v[SCAN_ITEMS];
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    const int64_t k = t0 + static_cast<int64_t>(threadIdx.x) * SCAN_ITEMS + i;
    v[i] = k < n ? in[k] : 0;
  }
  block_exclusive_scan(v, tile_off[blockIdx.x], ws);
  for (int i = 0; i < SCAN_ITEMS; ++i) {
    const int64_t k = t0 + static_cast<int64_t>(threadIdx.x) * SCAN_ITEMS + i;
    if (k < n) out[k] = v[i];
  }
}

}  // namespace csr
}  // namespace g2

namespace {
template <bool SCATTER>
int walk(const void* data, int32_t elem_bytes, const void* indices, const void* indptr, const void* offsets,
         int32_t index_bytes, int64_t n_elem, int32_t T, int32_t H, int32_t W, uint32_t* counter,
         const uint32_t* ev_off, int32_t* ev_times, void* ev_data, int32_t* err, void* stream) {
  using namespace g2;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const unsigned grid = static_cast<unsigned>(T < sms * 8 ? T : sms * 8);
  cudaStream_t st = as_stream(stream);
#define G2_WALK(TV, TI)                                                                                         \
  csr::walk_kernel<TV, TI, SCATTER><<<grid, csr::THREADS, 0, st>>>(                                             \
      reinterpret_cast<const TV*>(data), reinterpret_cast<const TI*>(indices), reinterpret_cast<const TI*>(indptr), \
      reinterpret_cast<const TI*>(offsets), n_elem, T, H, W, counter, ev_off, ev_times, reinterpret_cast<TV*>(ev_data), \
      err)
  if (elem_bytes == 1 && index_bytes == 4) G2_WALK(uint8_t, uint32_t);
  else if (elem_bytes == 1 && index_bytes == 8) G2_WALK(uint8_t, int64_t);
  else if (elem_bytes == 2 && index_bytes == 4) G2_WALK(uint16_t, uint32_t);
  else G2_WALK(uint16_t, int64_t);
#undef G2_WALK
  return launch_status();
}
}  // namespace

extern "C" int g2_csr_count(const void* indices_dev, const void* indptr_dev, const void* offsets_dev,
                            int32_t index_bytes, int64_t n_elem, int32_t nframes, int32_t height, int32_t width,
                            uint32_t* counts_dev, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!indices_dev || !indptr_dev || !offsets_dev || !counts_dev || !err_dev) return G2_ERR_ARG;
  if ((index_bytes != 4 && index_bytes != 8) || n_elem < 0 || nframes <= 0 || height <= 0 || width <= 0)
    return G2_ERR_ARG;
  return walk<false>(indices_dev, 1, indices_dev, indptr_dev, offsets_dev, index_bytes, n_elem, nframes, height,
                     width, counts_dev, nullptr, nullptr, nullptr, err_dev, stream);
}

extern "C" int g2_exclusive_scan_u32(const uint32_t* in_dev, int64_t n, uint32_t* out_dev, uint32_t* scratch_dev,
                                     int64_t scratch_len, void* stream) {
  using namespace g2;
  if (!in_dev || !out_dev || !scratch_dev || n <= 0) return G2_ERR_ARG;
  const int64_t n_tiles = (n + csr::SCAN_TILE - 1) / csr::SCAN_TILE;
  if (scratch_len < n_tiles) return G2_ERR_ARG;
  if (n_tiles > 0x7fffffff) return G2_ERR_TOO_LARGE;
  cudaStream_t st = as_stream(stream);
  csr::tile_sums_kernel<<<static_cast<unsigned>(n_tiles), csr::SCAN_THREADS, 0, st>>>(in_dev, n, scratch_dev);
  csr::scan_tile_sums_kernel<<<1, csr::SCAN_THREADS, 0, st>>>(scratch_dev, n_tiles, out_dev + n);
  csr::scan_tiles_kernel<<<static_cast<unsigned>(n_tiles), csr::SCAN_THREADS, 0, st>>>(in_dev, n, scratch_dev,
                                                                                     out_dev);
  return launch_status();
}

extern "C" int g2_csr_scatter(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                              const void* indptr_dev, const void* offsets_dev, int32_t index_bytes, int64_t n_elem,
                              int32_t nframes, int32_t height, int32_t width, const uint32_t* ev_offsets_dev,
                              uint32_t* cursor_dev, int32_t* ev_times_dev, void* ev_data_dev, int32_t* err_dev,
                              void* stream) {
  using namespace g2;
  if (!data_dev || !indices_dev || !indptr_dev || !offsets_dev || !ev_offsets_dev || !cursor_dev || !ev_times_dev ||
      !ev_data_dev || !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || (index_bytes != 4 && index_bytes != 8) || n_elem < 0 ||
      nframes <= 0 || height <= 0 || width <= 0)
    return G2_ERR_ARG;
  return walk<true>(data_dev, elem_bytes, indices_dev, indptr_dev, offsets_dev, index_bytes, n_elem, nframes,
                    height, width, cursor_dev, ev_offsets_dev, ev_times_dev, ev_data_dev, err_dev, stream);
}
