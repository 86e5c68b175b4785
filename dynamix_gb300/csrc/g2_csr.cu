// G7: per-frame CSR -> per-pixel event lists, so that the sparse correlator
// reuses the event pair-sum kernel (G6).
//
// CSR layout of dynamix's SparseCorrelator (intensity.py:70-77,
// correlator.cl:110-217): frame t owns elements [offsets[t], offsets[t+1]);
// indptr[t * (H+1) + r] .. indptr[t * (H+1) + r + 1] are the elements of row r
// relative to offsets[t]; indices[] is the column inside the row, data[] the
// count.  The transposition is a counting sort by pixel:
//   1. count   : events per pixel
//   2. scan    : exclusive prefix sum of the counts -> event offsets
//   3. scatter : each element goes to the slot of its pixel given by the
//                number of earlier frames holding that pixel.
// Row kernels (image rows up to ROW_MAX_W pixels): one warp owns one image row
// for all frames, its lanes take 32 consecutive frames at a time, and the
// per-pixel counters of the row live in the warp's shared memory, so neither
// pass needs a global atomic.  The scatter ranks the elements of a 32-frame
// batch per pixel with a bit mask (bit = frame of the batch), so every pixel's
// events come out in ascending frame order -- the layout FramesCompressor
// builds (event.py:267-284).  Wider rows use the walk kernels (a warp per row
// of a frame, global atomics, order inside a pixel unspecified).
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
      if (base < 0 || s < base || e < s || e > fend || e > n_elem) {
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

constexpr int ROW_MAX_W = 29000;       // 2 x W words of shared memory per warp in the scatter

// Counts of one image row over all frames (one warp per row).
template <typename Ti>
__global__ void __launch_bounds__(256)
    row_count_kernel(const Ti* __restrict__ indices, const Ti* __restrict__ indptr, const Ti* __restrict__ offsets,
                     int64_t n_elem, int32_t T, int32_t H, int32_t W, int rows_per_cta,
                     uint32_t* __restrict__ counts, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * rows_per_cta + warp;
  if (warp >= rows_per_cta || r >= H) return;  // warp-uniform; no block barrier below
  uint32_t* cnt = sm + static_cast<int64_t>(warp) * W;
  for (int i = lane; i < W; i += 32) cnt[i] = 0;
  __syncwarp();
  bool bad = false;
  for (int64_t t0 = 0; t0 < T; t0 += 32) {
    const int64_t t = t0 + lane;
    if (t >= T) continue;
    const int64_t base = static_cast<int64_t>(offsets[t]);
    const int64_t fend = static_cast<int64_t>(offsets[t + 1]);
    const Ti* ip = indptr + t * static_cast<int64_t>(H + 1) + r;
    const int64_t s = base + static_cast<int64_t>(ip[0]);
    const int64_t e = base + static_cast<int64_t>(ip[1]);
    if (base < 0 || s < base || e < s || e > fend || e > n_elem) {
      bad = true;
      continue;
    }
#pragma unroll 4
    for (int64_t k = s; k < e; ++k) {
      const int64_t col = static_cast<int64_t>(indices[k]);
      if (col < 0 || col >= W) {
        bad = true;
        continue;
      }
      atomicAdd(&cnt[col], 1u);
    }
  }
  __syncwarp();
  uint32_t* out = counts + static_cast<int64_t>(r) * W;
  for (int i = lane; i < W; i += 32)
    if (cnt[i]) out[i] += cnt[i];  // the row belongs to this warp alone
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Scatter of one image row over all frames, events of a pixel in frame order.
// A lane keeps the first KREG elements of its (frame, row) segment in
// registers across the three phases of a batch; longer segments reload the rest.
constexpr int KREG = 16;

template <typename Tv, typename Ti>
__global__ void __launch_bounds__(256)
    row_scatter_kernel(const Tv* __restrict__ data, const Ti* __restrict__ indices, const Ti* __restrict__ indptr,
                       const Ti* __restrict__ offsets, int64_t n_elem, int32_t T, int32_t H, int32_t W,
                       int rows_per_cta, const uint32_t* __restrict__ ev_off, int32_t* __restrict__ ev_times,
                       Tv* __restrict__ ev_data, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * rows_per_cta + warp;
  if (warp >= rows_per_cta || r >= H) return;  // warp-uniform; no block barrier below
  uint32_t* cur = sm + static_cast<int64_t>(warp) * 2 * W;  // next free slot of each pixel
  uint32_t* msk = cur + W;                                    // frames of the batch holding the pixel
  const uint32_t* row_off = ev_off + static_cast<int64_t>(r) * W;
  const uint32_t n_total = ev_off[static_cast<int64_t>(H) * W];
  for (int i = lane; i < W; i += 32) {
    cur[i] = row_off[i];
    msk[i] = 0;
  }
  __syncwarp();
  bool bad = false;
  const uint32_t bit = 1u << lane;
  for (int64_t t0 = 0; t0 < T; t0 += 32) {
    const int64_t t = t0 + lane;
    int64_t s = 0, e = 0;
    if (t < T) {
      const int64_t base = static_cast<int64_t>(offsets[t]);
      const int64_t fend = static_cast<int64_t>(offsets[t + 1]);
      const Ti* ip = indptr + t * static_cast<int64_t>(H + 1) + r;
      s = base + static_cast<int64_t>(ip[0]);
      e = base + static_cast<int64_t>(ip[1]);
      if (base < 0 || s < base || e < s || e > fend || e > n_elem) {
        bad = true;
        s = e = 0;
      }
    }
    const int len = static_cast<int>(e - s);
    int32_t col[KREG];
    Tv val[KREG];
    // 1. load the segment and mark the frames of the batch holding each pixel
#pragma unroll
    for (int j = 0; j < KREG; ++j) {
      col[j] = -1;
      if (j < len) {
        const int64_t c = static_cast<int64_t>(indices[s + j]);
        val[j] = data[s + j];
        col[j] = (c >= 0 && c < W) ? static_cast<int32_t>(c) : -1;  // bad columns: reported by the count pass
      }
    }
#pragma unroll
    for (int j = 0; j < KREG; ++j)
      if (col[j] >= 0 && (atomicOr(&msk[col[j]], bit) & bit)) bad = true;  // a column twice in one row
    for (int j = KREG; j < len; ++j) {
      const int64_t c = static_cast<int64_t>(indices[s + j]);
      if (c >= 0 && c < W && (atomicOr(&msk[c], bit) & bit)) bad = true;
    }
    __syncwarp();
    // 2. slot = next free slot + earlier frames of the batch holding the pixel
#pragma unroll
    for (int j = 0; j < KREG; ++j) {
      if (col[j] >= 0) {
        const uint32_t slot = cur[col[j]] + __popc(msk[col[j]] & (bit - 1u));
        if (slot < n_total) {
          ev_times[slot] = static_cast<int32_t>(t);
          ev_data[slot] = val[j];
        } else {
          bad = true;
        }
      }
    }
    for (int j = KREG; j < len; ++j) {
      const int64_t c = static_cast<int64_t>(indices[s + j]);
      if (c < 0 || c >= W) continue;
      const uint32_t slot = cur[c] + __popc(msk[c] & (bit - 1u));
      if (slot < n_total) {
        ev_times[slot] = static_cast<int32_t>(t);
        ev_data[slot] = data[s + j];
      } else {
        bad = true;
      }
    }
    __syncwarp();
    // 3. the last frame of the batch holding the pixel advances its cursor
#pragma unroll
    for (int j = 0; j < KREG; ++j) {
      if (col[j] >= 0) {
        const uint32_t m = msk[col[j]];
        if (m != 0u && (m >> lane) == 1u) {
          cur[col[j]] += __popc(m);
          msk[col[j]] = 0u;
        }
      }
    }
    for (int j = KREG; j < len; ++j) {
      const int64_t c = static_cast<int64_t>(indices[s + j]);
      if (c < 0 || c >= W) continue;
      const uint32_t m = msk[c];
      if (m != 0u && (m >> lane) == 1u) {
        cur[c] += __popc(m);
        msk[c] = 0u;
      }
    }
    __syncwarp();
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Frame order inside each pixel's list of packed words that is already ordered
// by 32-frame window (t >> 5): a warp per pixel takes 32 words at a time and
// ranks each word inside its window group by shuffles; a group that may run on
// past the 32 words waits for the next round.
__global__ void __launch_bounds__(256)
    sort_windows_kernel(uint32_t* __restrict__ words, const uint32_t* __restrict__ ev_off, int64_t npix) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
  for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x >> 5) + (threadIdx.x >> 5); p < npix;
       p += warps) {
    const int64_t s = ev_off[p];
    const int64_t n = static_cast<int64_t>(ev_off[p + 1]) - s;
    int64_t c0 = 0;
    while (c0 + 1 < n) {
      const bool has = c0 + lane < n;
      const uint32_t w = has ? words[s + c0 + lane] : 0xFFFFFFFFu;
      const uint32_t win = has ? (w >> 21) : 0xFFFFFFFFu;          // (t >> 5)
      const uint32_t prev_win = __shfl_up_sync(0xffffffffu, win, 1);
      const uint32_t heads = __ballot_sync(0xffffffffu, has && (lane == 0 || win != prev_win));
      const int avail = static_cast<int>(n - c0 < 32 ? n - c0 : 32);
      int commit = avail;
      if (c0 + 32 < n) {                                            // the last group may continue
        const int last_head = 31 - __clz(heads);
        commit = last_head > 0 ? last_head : 32;
      }
      const uint32_t le = heads & (lane == 31 ? 0xffffffffu : ((2u << lane) - 1u));
      const int start = le ? 31 - __clz(le) : 0;
      const uint32_t gt = heads & ~(lane == 31 ? 0xffffffffu : ((2u << lane) - 1u));
      const int gend = min(gt ? __ffs(gt) - 1 : 32, commit);
      const uint32_t t = w >> 16;
      int rank = 0;
      for (int j = 0; j < 32; ++j) {
        const uint32_t tj = __shfl_sync(0xffffffffu, t, j);
        rank += (j >= start && j < gend && (tj < t || (tj == t && j < lane))) ? 1 : 0;
      }
      __syncwarp();
      if (lane < commit) words[s + c0 + start + rank] = w;
      __syncwarp();
      c0 += commit;
    }
  }
}

// Sub-blocked transposition (frames < 2^16): the frames are cut into
// sub-blocks of SUBBLOCK frames.  The count pass keeps, per image row (one
// warp, lanes = 32 consecutive frames), the per-pixel counts of each
// sub-block (uint16) instead of one total.  The scatter runs one CTA per (8
// consecutive sub-blocks, image row), a warp per sub-block with its own slot
// cursors (the pixel's offset plus the counts of the earlier sub-blocks), so
// the CTA writes, for every pixel of its row, one contiguous stretch of that
// pixel's list (8 x 1024 frames of events) while it runs: the sectors it
// fills are complete before they leave L2.  Events come out ordered by
// 32-frame window within a pixel, in any order inside a window.
constexpr int SUBBLOCK = 1024;
constexpr int SB_PER_CTA = 8;

// Row bounds transposed to row-major: rb[r * T + t] = offsets[t] + indptr[t][r]
// (absolute element index of the start of row r in frame t; r = H is the
// frame's end), so that a warp walking one row over 32 consecutive frames
// reads its bounds with one coalesced load.  Malformed pointers are reported
// and replaced by an empty row.
template <typename Ti>
__global__ void __launch_bounds__(256)
    row_bounds_kernel(const Ti* __restrict__ indptr, const Ti* __restrict__ offsets, int64_t n_elem, int32_t T,
                      int32_t H, uint32_t* __restrict__ rb, int32_t* __restrict__ err) {
  __shared__ uint32_t tile[32][33];
  const int64_t t0 = static_cast<int64_t>(blockIdx.x) * 32, r0 = static_cast<int64_t>(blockIdx.y) * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
  bool bad = false;
  for (int k = ty; k < 32; k += 8) {
    const int64_t t = t0 + k, r = r0 + tx;
    uint32_t v = 0;
    if (t < T && r <= H) {
      const int64_t base = static_cast<int64_t>(offsets[t]);
      const int64_t fend = static_cast<int64_t>(offsets[t + 1]);
      const int64_t a = base + static_cast<int64_t>(indptr[t * static_cast<int64_t>(H + 1) + r]);
      if (base < 0 || a < base || a > fend || fend > n_elem) {
        bad = true;
        v = static_cast<uint32_t>(base < 0 ? 0 : (base > n_elem ? n_elem : base));
      } else {
        v = static_cast<uint32_t>(a);
      }
    }
    tile[k][tx] = v;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r0 + k, t = t0 + tx;
    if (t < T && r <= H) rb[r * T + t] = tile[tx][k];
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

template <typename Ti>
__global__ void __launch_bounds__(256)
    row_count_blocked_kernel(const Ti* __restrict__ indices, const uint32_t* __restrict__ rb, int64_t n_elem,
                             int32_t T, int32_t H, int32_t W, int rows_per_cta, uint16_t* __restrict__ sb_counts,
                             int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.x * rows_per_cta + warp;
  if (warp >= rows_per_cta || r >= H) return;  // warp-uniform; no block barrier below
  uint32_t* cnt = sm + static_cast<int64_t>(warp) * W;
  for (int i = lane; i < W; i += 32) cnt[i] = 0;
  __syncwarp();
  const int64_t npix = static_cast<int64_t>(H) * W;
  bool bad = false;
  for (int64_t sb0 = 0; sb0 < T; sb0 += SUBBLOCK) {
    const int64_t sb_end = sb0 + SUBBLOCK < T ? sb0 + SUBBLOCK : T;
    for (int64_t t0 = sb0; t0 < sb_end; t0 += 32) {
      const int64_t t = t0 + lane;
      if (t >= sb_end) continue;
      const int64_t s = rb[static_cast<int64_t>(r) * T + t];
      const int64_t e = rb[static_cast<int64_t>(r + 1) * T + t];
      if (e < s || e > n_elem) {
        bad = true;
        continue;
      }
      int64_t prev = -1;
#pragma unroll 4
      for (int64_t k = s; k < e; ++k) {
        const int64_t col = static_cast<int64_t>(indices[k]);
        bad |= col <= prev;  // repeated or descending column (sorted CSR expected)
        prev = col;
        if (col < 0 || col >= W) {
          bad = true;
          continue;
        }
        atomicAdd(&cnt[col], 1u);
      }
    }
    __syncwarp();
    uint16_t* out = sb_counts + (sb0 / SUBBLOCK) * npix + static_cast<int64_t>(r) * W;
    for (int i = lane; i < W; i += 32) {
      out[i] = static_cast<uint16_t>(cnt[i]);  // <= SUBBLOCK frames, one element each
      cnt[i] = 0;
    }
    __syncwarp();
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// counts[p] += sum over sub-blocks of sb_counts[sb][p]
__global__ void __launch_bounds__(256)
    sum_subblocks_kernel(const uint16_t* __restrict__ sb_counts, int n_sb, int64_t npix,
                         uint32_t* __restrict__ counts) {
  for (int64_t p = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; p < npix;
       p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    uint32_t s = 0;
    for (int b = 0; b < n_sb; ++b) s += sb_counts[b * npix + p];
    counts[p] += s;
  }
}

template <typename Tv, typename Ti>
__global__ void __launch_bounds__(SB_PER_CTA * 32)
    row_scatter_blocked_kernel(const Tv* __restrict__ data, const Ti* __restrict__ indices,
                               const uint32_t* __restrict__ rb, int64_t n_elem, int32_t T, int32_t H, int32_t W,
                               const uint32_t* __restrict__ ev_off, const uint16_t* __restrict__ sb_counts,
                               uint32_t* __restrict__ ev_words, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r = blockIdx.y;
  const int64_t sb = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + warp;
  const int64_t sb0 = sb * SUBBLOCK;
  if (r >= H || sb0 >= T) return;  // warp-uniform; no block barrier below
  const int64_t npix = static_cast<int64_t>(H) * W;
  uint32_t* cur = sm + static_cast<int64_t>(warp) * W;
  const int64_t row0 = static_cast<int64_t>(r) * W;
  // the sub-block's first slot of each pixel: its offset plus the earlier sub-blocks
  for (int i = lane; i < W; i += 32) {
    uint32_t c = ev_off[row0 + i];
#pragma unroll 8
    for (int64_t b = 0; b < sb; ++b) c += sb_counts[b * npix + row0 + i];
    cur[i] = c;
  }
  __syncwarp();
  const uint32_t n_total = ev_off[npix];
  const int64_t sb_end = sb0 + SUBBLOCK < T ? sb0 + SUBBLOCK : T;
  // per batch of 32 frames, the lanes' segments (lane = frame) are walked as
  // one flattened list, lane x taking element x: consecutive lanes read
  // consecutive elements of a segment instead of 32 segments at once
  uint32_t* pre = sm + static_cast<int64_t>(blockDim.x >> 5) * W + warp * 66;  // [33] exclusive prefix
  uint32_t* beg = pre + 33;                                                    // [32] segment starts
  bool bad = false;
  for (int64_t t0 = sb0; t0 < sb_end; t0 += 32) {
    const int64_t t = t0 + lane;
    int64_t s = 0, e = 0;
    if (t < sb_end) {
      s = rb[static_cast<int64_t>(r) * T + t];
      e = rb[static_cast<int64_t>(r + 1) * T + t];
      if (e < s || e > n_elem) {
        bad = true;
        s = e = 0;
      }
    }
    const uint32_t len = static_cast<uint32_t>(e - s);
    uint32_t incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    pre[lane] = incl - len;
    if (lane == 31) pre[32] = total;
    beg[lane] = static_cast<uint32_t>(s);
    __syncwarp();
    for (uint32_t x = lane; x < total; x += 32) {
      int f = 0;  // the last frame whose segment starts at or before x
#pragma unroll
      for (int step = 16; step; step >>= 1)
        if (pre[f + step] <= x) f += step;
      const int64_t k = static_cast<int64_t>(beg[f]) + (x - pre[f]);
      const int64_t c = static_cast<int64_t>(indices[k]);
      if (c < 0 || c >= W) {
        bad = true;
        continue;
      }
      const uint32_t slot = atomicAdd(&cur[c], 1u);
      if (slot < n_total)
        ev_words[slot] = (static_cast<uint32_t>(t0 + f) << 16) | static_cast<uint32_t>(data[k]);
      else
        bad = true;
    }
    __syncwarp();  // pre/beg are rewritten by the next batch
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Packed words -> (times int32, data) arrays.
template <typename Tv>
__global__ void __launch_bounds__(256)
    unpack_events_kernel(const uint32_t* __restrict__ words, int64_t n, int32_t* __restrict__ times,
                         Tv* __restrict__ data) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const uint32_t w = words[i];
    times[i] = static_cast<int32_t>(w >> 16);
    data[i] = static_cast<Tv>(w & 0xFFFFu);
  }
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

namespace {
// Warps (image rows) per CTA so that a CTA holds about 64 KB of row counters.
int rows_per_cta(int32_t W, int words_per_px) {
  const int64_t per_row = static_cast<int64_t>(W) * words_per_px * 4;
  int64_t r = 65536 / per_row;
  return static_cast<int>(r < 1 ? 1 : (r > 8 ? 8 : r));
}

template <typename K>
bool allow_smem(K kernel, int64_t bytes) {
  if (bytes <= 48 * 1024) return true;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)) ==
         cudaSuccess;
}

int row_count(const void* indices, const void* indptr, const void* offsets, int32_t index_bytes, int64_t n_elem,
              int32_t T, int32_t H, int32_t W, uint32_t* counts, int32_t* err, void* stream) {
  using namespace g2;
  const int rpc = rows_per_cta(W, 1);
  const int64_t smem = static_cast<int64_t>(rpc) * W * 4;
  const unsigned grid = static_cast<unsigned>((H + rpc - 1) / rpc);
  cudaStream_t st = as_stream(stream);
  if (index_bytes == 4) {
    if (!allow_smem(csr::row_count_kernel<uint32_t>, smem)) return G2_ERR_CUDA;
    csr::row_count_kernel<uint32_t><<<grid, rpc * 32, smem, st>>>(
        reinterpret_cast<const uint32_t*>(indices), reinterpret_cast<const uint32_t*>(indptr),
        reinterpret_cast<const uint32_t*>(offsets), n_elem, T, H, W, rpc, counts, err);
  } else {
    if (!allow_smem(csr::row_count_kernel<int64_t>, smem)) return G2_ERR_CUDA;
    csr::row_count_kernel<int64_t><<<grid, rpc * 32, smem, st>>>(
        reinterpret_cast<const int64_t*>(indices), reinterpret_cast<const int64_t*>(indptr),
        reinterpret_cast<const int64_t*>(offsets), n_elem, T, H, W, rpc, counts, err);
  }
  return launch_status();
}

template <typename Tv, typename Ti>
int row_scatter_t(const void* data, const void* indices, const void* indptr, const void* offsets, int64_t n_elem,
                  int32_t T, int32_t H, int32_t W, const uint32_t* ev_off, int32_t* ev_times, void* ev_data,
                  int32_t* err, cudaStream_t st) {
  using namespace g2;
  const int rpc = rows_per_cta(W, 2);
  const int64_t smem = static_cast<int64_t>(rpc) * W * 8;
  const unsigned grid = static_cast<unsigned>((H + rpc - 1) / rpc);
  if (!allow_smem(csr::row_scatter_kernel<Tv, Ti>, smem)) return G2_ERR_CUDA;
  csr::row_scatter_kernel<Tv, Ti><<<grid, rpc * 32, smem, st>>>(
      reinterpret_cast<const Tv*>(data), reinterpret_cast<const Ti*>(indices), reinterpret_cast<const Ti*>(indptr),
      reinterpret_cast<const Ti*>(offsets), n_elem, T, H, W, rpc, ev_off, ev_times, reinterpret_cast<Tv*>(ev_data),
      err);
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
  if (width <= csr::ROW_MAX_W)
    return row_count(indices_dev, indptr_dev, offsets_dev, index_bytes, n_elem, nframes, height, width, counts_dev,
                     err_dev, stream);
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
  if (width <= csr::ROW_MAX_W) {
    cudaStream_t st = as_stream(stream);
    if (elem_bytes == 1 && index_bytes == 4)
      return row_scatter_t<uint8_t, uint32_t>(data_dev, indices_dev, indptr_dev, offsets_dev, n_elem, nframes, height,
                                              width, ev_offsets_dev, ev_times_dev, ev_data_dev, err_dev, st);
    if (elem_bytes == 1)
      return row_scatter_t<uint8_t, int64_t>(data_dev, indices_dev, indptr_dev, offsets_dev, n_elem, nframes, height,
                                             width, ev_offsets_dev, ev_times_dev, ev_data_dev, err_dev, st);
    if (index_bytes == 4)
      return row_scatter_t<uint16_t, uint32_t>(data_dev, indices_dev, indptr_dev, offsets_dev, n_elem, nframes,
                                               height, width, ev_offsets_dev, ev_times_dev, ev_data_dev, err_dev, st);
    return row_scatter_t<uint16_t, int64_t>(data_dev, indices_dev, indptr_dev, offsets_dev, n_elem, nframes, height,
                                            width, ev_offsets_dev, ev_times_dev, ev_data_dev, err_dev, st);
  }
  return walk<true>(data_dev, elem_bytes, indices_dev, indptr_dev, offsets_dev, index_bytes, n_elem, nframes,
                    height, width, cursor_dev, ev_offsets_dev, ev_times_dev, ev_data_dev, err_dev, stream);
}

extern "C" int g2_csr_count_blocked(const void* indices_dev, const void* indptr_dev, const void* offsets_dev,
                                    int32_t index_bytes, int64_t n_elem, int32_t nframes, int32_t height,
                                    int32_t width, uint32_t* row_bounds_dev, uint32_t* counts_dev,
                                    uint16_t* sb_counts_dev, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!indices_dev || !indptr_dev || !offsets_dev || !row_bounds_dev || !counts_dev || !sb_counts_dev || !err_dev)
    return G2_ERR_ARG;
  if ((index_bytes != 4 && index_bytes != 8) || n_elem < 0 || nframes <= 0 || height <= 0 || width <= 0)
    return G2_ERR_ARG;
  if (width > csr::ROW_MAX_W || n_elem >= (1ll << 32)) return G2_ERR_UNSUPPORTED;
  cudaStream_t st = as_stream(stream);
  const dim3 tgrid(static_cast<unsigned>((nframes + 31) / 32), static_cast<unsigned>((height + 1 + 31) / 32));
  if (index_bytes == 4)
    csr::row_bounds_kernel<uint32_t><<<tgrid, 256, 0, st>>>(reinterpret_cast<const uint32_t*>(indptr_dev),
                                                             reinterpret_cast<const uint32_t*>(offsets_dev), n_elem,
                                                             nframes, height, row_bounds_dev, err_dev);
  else
    csr::row_bounds_kernel<int64_t><<<tgrid, 256, 0, st>>>(reinterpret_cast<const int64_t*>(indptr_dev),
                                                            reinterpret_cast<const int64_t*>(offsets_dev), n_elem,
                                                            nframes, height, row_bounds_dev, err_dev);
  const int rpc = rows_per_cta(width, 1);
  const int64_t smem = static_cast<int64_t>(rpc) * width * 4;
  const unsigned grid = static_cast<unsigned>((height + rpc - 1) / rpc);
  if (index_bytes == 4) {
    if (!allow_smem(csr::row_count_blocked_kernel<uint32_t>, smem)) return G2_ERR_CUDA;
    csr::row_count_blocked_kernel<uint32_t><<<grid, rpc * 32, smem, st>>>(
        reinterpret_cast<const uint32_t*>(indices_dev), row_bounds_dev, n_elem, nframes, height, width, rpc,
        sb_counts_dev, err_dev);
  } else {
    if (!allow_smem(csr::row_count_blocked_kernel<int64_t>, smem)) return G2_ERR_CUDA;
    csr::row_count_blocked_kernel<int64_t><<<grid, rpc * 32, smem, st>>>(
        reinterpret_cast<const int64_t*>(indices_dev), row_bounds_dev, n_elem, nframes, height, width, rpc,
        sb_counts_dev, err_dev);
  }
  const int64_t npix = static_cast<int64_t>(height) * width;
  const int n_sb = static_cast<int>((static_cast<int64_t>(nframes) + csr::SUBBLOCK - 1) / csr::SUBBLOCK);
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  int64_t blocks = (npix + 255) / 256;
  if (blocks > static_cast<int64_t>(sms) * 16) blocks = static_cast<int64_t>(sms) * 16;
  csr::sum_subblocks_kernel<<<static_cast<unsigned>(blocks), 256, 0, st>>>(sb_counts_dev, n_sb, npix, counts_dev);
  return launch_status();
}

extern "C" int g2_csr_scatter_blocked(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                                      const uint32_t* row_bounds_dev, int32_t index_bytes, int64_t n_elem,
                                      int32_t nframes, int32_t height, int32_t width, const uint32_t* ev_offsets_dev,
                                      const uint16_t* sb_counts_dev, uint32_t* ev_words_dev, int32_t* err_dev,
                                      void* stream) {
  using namespace g2;
  if (!data_dev || !indices_dev || !row_bounds_dev || !ev_offsets_dev || !sb_counts_dev || !ev_words_dev ||
      !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || (index_bytes != 4 && index_bytes != 8) || n_elem < 0 ||
      nframes <= 0 || height <= 0 || width <= 0)
    return G2_ERR_ARG;
  if (nframes > 65536 || width > csr::ROW_MAX_W || n_elem >= (1ll << 32)) return G2_ERR_UNSUPPORTED;
  // warps (sub-blocks) per CTA: up to 8, each holding one row of cursors
  int warps = static_cast<int>((227 * 1024) / (static_cast<int64_t>(width) * 4 + 66 * 4));
  warps = warps < 1 ? 1 : (warps > csr::SB_PER_CTA ? csr::SB_PER_CTA : warps);
  const int64_t smem = static_cast<int64_t>(warps) * (width + 66) * 4;
  const int64_t n_sb = (static_cast<int64_t>(nframes) + csr::SUBBLOCK - 1) / csr::SUBBLOCK;
  const dim3 grid(static_cast<unsigned>((n_sb + warps - 1) / warps), static_cast<unsigned>(height));
  cudaStream_t st = as_stream(stream);
#define G2_BS(TV, TI)                                                                                           \
  do {                                                                                                          \
    if (!allow_smem(csr::row_scatter_blocked_kernel<TV, TI>, smem)) return G2_ERR_CUDA;                         \
    csr::row_scatter_blocked_kernel<TV, TI><<<grid, warps * 32, smem, st>>>(                                    \
        reinterpret_cast<const TV*>(data_dev), reinterpret_cast<const TI*>(indices_dev), row_bounds_dev, n_elem, \
        nframes, height, width, ev_offsets_dev, sb_counts_dev, ev_words_dev, err_dev);                          \
  } while (0)
  if (elem_bytes == 1 && index_bytes == 4) G2_BS(uint8_t, uint32_t);
  else if (elem_bytes == 1) G2_BS(uint8_t, int64_t);
  else if (index_bytes == 4) G2_BS(uint16_t, uint32_t);
  else G2_BS(uint16_t, int64_t);
#undef G2_BS
  return launch_status();
}

extern "C" int g2_events_sort_windows(uint32_t* ev_words_dev, const uint32_t* ev_offsets_dev, int64_t npix,
                                      void* stream) {
  using namespace g2;
  if (!ev_words_dev || !ev_offsets_dev || npix <= 0) return G2_ERR_ARG;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  int64_t blocks = (npix + 7) / 8;
  if (blocks > static_cast<int64_t>(sms) * 16) blocks = static_cast<int64_t>(sms) * 16;
  csr::sort_windows_kernel<<<static_cast<unsigned>(blocks), 256, 0, as_stream(stream)>>>(ev_words_dev,
                                                                                       ev_offsets_dev, npix);
  return launch_status();
}

extern "C" int g2_events_unpack(const uint32_t* ev_words_dev, int64_t n_events, int32_t elem_bytes,
                                int32_t* ev_times_dev, void* ev_data_dev, void* stream) {
  using namespace g2;
  if (!ev_words_dev || !ev_times_dev || !ev_data_dev || n_events < 0 || (elem_bytes != 1 && elem_bytes != 2))
    return G2_ERR_ARG;
  if (n_events == 0) return G2_OK;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  int64_t blocks = (n_events + 255) / 256;
  if (blocks > static_cast<int64_t>(sms) * 16) blocks = static_cast<int64_t>(sms) * 16;
  cudaStream_t st = as_stream(stream);
  if (elem_bytes == 1)
    csr::unpack_events_kernel<uint8_t><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
        ev_words_dev, n_events, ev_times_dev, reinterpret_cast<uint8_t*>(ev_data_dev));
  else
    csr::unpack_events_kernel<uint16_t><<<static_cast<unsigned>(blocks), 256, 0, st>>>(
        ev_words_dev, n_events, ev_times_dev, reinterpret_cast<uint16_t*>(ev_data_dev));
  return launch_status();
}
