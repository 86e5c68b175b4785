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

// Sub-blocked transposition (frames < 2^16, fewer than 2^32 elements): the
// frames are cut into sub-blocks of SUBBLOCK frames.  The count pass keeps,
// per image row (one warp, lanes = 32 consecutive frames), the per-pixel
// counts of each sub-block (uint16) and the row's total per sub-block.  The
// stage pass (one CTA per sub-block and row) writes the row's elements of the
// sub-block into one contiguous stretch of a staging area, pixel by pixel; the
// gather pass copies every pixel's runs, sub-block after sub-block, into the
// pixel's list.  Each pass writes inside regions that stay in L2 until they
// are complete (a single-pass scatter, whose every warp holds one partly
// written sector per pixel of its row for 1024 frames, moves several times
// its bytes through DRAM).
constexpr int SUBBLOCK = 1024;
constexpr int TILE_P = 64;  // pixels of one gather tile
constexpr int STAGE_THREADS = 512;  // threads of a stage CTA (the shared region limits CTAs per SM)
constexpr int UNROLL = 4;   // elements per lane with loads in flight together

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

// Count pass: one CTA per (sub-block, image row), the row's per-pixel counters
// in shared memory.  Warps take 32-frame batches and walk each batch's
// segments as one flattened list (lane x takes element x, so consecutive
// lanes read consecutive indices); a column not above its predecessor in the
// same segment is reported (sorted CSR expected).
template <typename Ti>
__global__ void __launch_bounds__(256)
    row_count_blocked_kernel(const Ti* __restrict__ indices, const uint32_t* __restrict__ rb, int64_t n_elem,
                             int32_t T, int32_t H, int32_t W, uint16_t* __restrict__ sb_counts,
                             uint32_t* __restrict__ row_totals, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  __shared__ uint32_t s_tot[8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sb = blockIdx.x;
  const int r = blockIdx.y;
  const int64_t sb0 = sb * SUBBLOCK;
  const int64_t sb_end = sb0 + SUBBLOCK < T ? sb0 + SUBBLOCK : T;
  uint32_t* cnt = sm;                  // [W] elements of each pixel of the row
  uint32_t* pre = sm + W + warp * 66;  // [33] exclusive prefix of a batch's segments
  uint32_t* beg = pre + 33;            // [32] segment starts
  for (int i = threadIdx.x; i < W; i += 256) cnt[i] = 0;
  __syncthreads();
  bool bad = false;
  for (int64_t t0 = sb0 + warp * 32; t0 < sb_end; t0 += 8 * 32) {
    const int64_t t = t0 + lane;
    int64_t a = 0, b = 0;
    if (t < sb_end) {
      a = rb[static_cast<int64_t>(r) * T + t];
      b = rb[static_cast<int64_t>(r + 1) * T + t];
      if (b < a || b > n_elem) {
        bad = true;
        a = b = 0;
      }
    }
    const uint32_t len = static_cast<uint32_t>(b - a);
    uint32_t inc = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    pre[lane] = inc - len;
    if (lane == 31) pre[32] = total;
    beg[lane] = static_cast<uint32_t>(a);
    __syncwarp();
    for (uint32_t x0 = 0; x0 < total; x0 += 32 * UNROLL) {
      int64_t c[UNROLL], prev[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const uint32_t x = x0 + u * 32 + lane;
        c[u] = -1;
        prev[u] = -2;
        if (x < total) {
          int f = 0;  // the last frame whose segment starts at or before x
#pragma unroll
          for (int step = 16; step; step >>= 1)
            if (pre[f + step] <= x) f += step;
          const int64_t k = static_cast<int64_t>(beg[f]) + (x - pre[f]);
          c[u] = static_cast<int64_t>(indices[k]);
          if (x > pre[f]) prev[u] = static_cast<int64_t>(indices[k - 1]);
        }
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        if (x0 + u * 32 + lane >= total) continue;
        bad |= c[u] <= prev[u];  // repeated or descending column
        if (c[u] < 0 || c[u] >= W) {
          bad = true;
          continue;
        }
        atomicAdd(&cnt[c[u]], 1u);
      }
    }
    __syncwarp();  // pre/beg are rewritten by the next batch
  }
  __syncthreads();
  uint16_t* out = sb_counts + sb * (static_cast<int64_t>(H) * W) + static_cast<int64_t>(r) * W;
  uint32_t tot = 0;
  for (int i = threadIdx.x; i < W; i += 256) {
    const uint16_t v = static_cast<uint16_t>(cnt[i]);  // <= SUBBLOCK frames, one element each
    out[i] = v;
    tot += v;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(0xffffffffu, tot, o);
  if (lane == 0) s_tot[warp] = tot;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t sum = 0;
    for (int w = 0; w < 8; ++w) sum += s_tot[w];
    row_totals[sb * H + r] = sum;
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

// Stage pass: one CTA per (sub-block, image row).  The row's elements of the
// sub-block go to a staging area ordered sub-block by sub-block, row by row and
// pixel by pixel; within a sub-block the staging area is therefore the
// exclusive scan of sb_counts in pixel order.  The CTA assembles its region in
// shared memory when it fits in buf_words and writes it out with coalesced
// stores (no partly written sector leaves the SM); a larger region is written
// in place.  Warps take 32-frame batches and walk each batch's segments as one
// flattened list (lane x takes element x).  The start of every TILE_P-pixel
// tile of the sub-block goes to tile_pos[sb * n_tiles + tile] for the gather.
template <typename Tv, typename Ti>
__global__ void __launch_bounds__(STAGE_THREADS)
    row_stage_kernel(const Tv* __restrict__ data, const Ti* __restrict__ indices, const uint32_t* __restrict__ rb,
                     int64_t n_elem, int32_t T, int32_t H, int32_t W, const uint16_t* __restrict__ sb_counts,
                     const uint32_t* __restrict__ row_base, int64_t n_tiles, uint32_t* __restrict__ tile_pos,
                     int buf_words, uint32_t* __restrict__ stage, int32_t frame0, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  __shared__ uint32_t s_tot[STAGE_THREADS / 32];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t sb = blockIdx.x;
  const int r = blockIdx.y;
  const int64_t npix = static_cast<int64_t>(H) * W;
  const int64_t sb0 = sb * SUBBLOCK;
  const int64_t sb_end = sb0 + SUBBLOCK < T ? sb0 + SUBBLOCK : T;
  uint32_t* cur = sm;                  // [W] next slot of each pixel, relative to the region
  uint32_t* pre = sm + W + warp * 66;  // [33] exclusive prefix of a batch's segments
  uint32_t* beg = pre + 33;            // [32] segment starts
  uint32_t* buf = sm + W + (STAGE_THREADS / 32) * 66;  // [buf_words] the region
  const uint16_t* cnt = sb_counts + sb * npix + static_cast<int64_t>(r) * W;
  // exclusive scan of the row's counts, each thread over a contiguous span
  const int per = (W + STAGE_THREADS - 1) / STAGE_THREADS;
  const int i0 = threadIdx.x * per, i1 = min(W, i0 + per);
  uint32_t own = 0;
  for (int i = i0; i < i1; ++i) own += cnt[i];
  uint32_t incl = own;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_tot[warp] = incl;
  __syncthreads();
  uint32_t run = incl - own, total = 0;
  for (int w = 0; w < STAGE_THREADS / 32; ++w) {
    run += w < warp ? s_tot[w] : 0u;
    total += s_tot[w];
  }
  const int64_t base = row_base[sb * H + r];
  const int64_t pix0 = static_cast<int64_t>(r) * W;
  for (int i = i0; i < i1; ++i) {
    cur[i] = run;
    if ((pix0 + i) % TILE_P == 0) tile_pos[sb * n_tiles + (pix0 + i) / TILE_P] = static_cast<uint32_t>(base + run);
    run += cnt[i];
  }
  __syncthreads();
  const bool skip = base + total > n_elem;  // block-uniform
  bool bad = skip;
  const bool buffered = total <= static_cast<uint32_t>(buf_words);
  for (int64_t t0 = sb0 + warp * 32; t0 < sb_end && !skip; t0 += STAGE_THREADS) {
    const int64_t t = t0 + lane;
    int64_t a = 0, b = 0;
    if (t < sb_end) {
      a = rb[static_cast<int64_t>(r) * T + t];
      b = rb[static_cast<int64_t>(r + 1) * T + t];
      if (b < a || b > n_elem) {
        bad = true;
        a = b = 0;
      }
    }
    const uint32_t len = static_cast<uint32_t>(b - a);
    uint32_t inc = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    const uint32_t seg_total = __shfl_sync(0xffffffffu, inc, 31);
    pre[lane] = inc - len;
    if (lane == 31) pre[32] = seg_total;
    beg[lane] = static_cast<uint32_t>(a);
    __syncwarp();
    for (uint32_t x0 = 0; x0 < seg_total; x0 += 32 * UNROLL) {
      // the loads of UNROLL elements are issued before their shared-memory
      // atomics, so every lane keeps several global loads in flight
      int64_t c[UNROLL];
      uint32_t w[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const uint32_t x = x0 + u * 32 + lane;
        c[u] = -1;
        w[u] = 0;
        if (x < seg_total) {
          int f = 0;  // the last frame whose segment starts at or before x
#pragma unroll
          for (int step = 16; step; step >>= 1)
            if (pre[f + step] <= x) f += step;
          const int64_t k = static_cast<int64_t>(beg[f]) + (x - pre[f]);
          c[u] = static_cast<int64_t>(indices[k]);
          w[u] = (static_cast<uint32_t>(frame0 + t0 + f) << 16) | static_cast<uint32_t>(data[k]);
        }
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        if (x0 + u * 32 + lane >= seg_total) continue;
        if (c[u] < 0 || c[u] >= W) {
          bad = true;
          continue;
        }
        const uint32_t slot = atomicAdd(&cur[c[u]], 1u);
        if (slot >= total)
          bad = true;
        else if (buffered)
          buf[slot] = w[u];
        else
          stage[base + slot] = w[u];
      }
    }
    __syncwarp();  // pre/beg are rewritten by the next batch
  }
  if (buffered && !skip) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < total; i += STAGE_THREADS) stage[base + i] = buf[i];
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Gather pass: one CTA per tile of TILE_P consecutive pixels.  For every
// sub-block the tile's runs are one contiguous chunk of the staging area
// (starting at tile_pos).  A thread per (sub-block, pixel) run copies the run
// to its pixel's list position in a shared-memory copy of the tile's part of
// the event lists (when it fits in buf_words, else in place), and the CTA
// writes that out with coalesced stores.  With `sort`, each run (one pixel,
// one 1024-frame sub-block) is put in frame order by insertion, which gives
// exactly the FramesCompressor layout.  Shared memory: 131 * n_sb + 1 words of
// tables, then the buffer.
// Output modes of the gather: the staged words as they are (CSR path, absolute
// frame numbers below 2^16), words whose frame field is relative to the
// sub-block (frame compression) turned into absolute packed words, or split
// into frame numbers (int32) and values (Tv).
constexpr int GATHER_WORDS = 0;
constexpr int GATHER_REL_WORDS = 1;
constexpr int GATHER_REL_SPLIT = 2;

template <int MODE, typename Tv>
__global__ void __launch_bounds__(256)
    gather_tiles_kernel(const uint32_t* __restrict__ stage, const uint32_t* __restrict__ tile_pos,
                        const uint16_t* __restrict__ sb_counts, int n_sb, int64_t npix, int64_t n_tiles,
                        const uint32_t* __restrict__ ev_off, int64_t n_elem, int sort, int buf_words,
                        int warp_runs, uint32_t* __restrict__ ev_words, int32_t* __restrict__ ev_times,
                        Tv* __restrict__ ev_data, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  uint32_t* cp = sm;                       // [n_sb][TILE_P + 1] run starts within each chunk
  uint32_t* dst = cp + n_sb * (TILE_P + 1);  // [n_sb][TILE_P] run starts within the tile's lists
  uint32_t* cb = dst + n_sb * TILE_P;        // [n_sb + 1] chunk starts within the walk
  uint32_t* tp = cb + n_sb + 1;              // [n_sb] chunk starts in the staging area
  uint32_t* buf = tp + n_sb;                 // [buf_words] words, or frame numbers
  uint16_t* bufd = reinterpret_cast<uint16_t*>(buf + buf_words);  // [buf_words] values (split mode)
  __shared__ int s_bad;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile = blockIdx.x;
  const int64_t p0 = tile * TILE_P;
  const int np = static_cast<int>(npix - p0 < TILE_P ? npix - p0 : TILE_P);
  const int64_t base = ev_off[p0];
  const int64_t tile_total = static_cast<int64_t>(ev_off[p0 + np]) - base;
  if (threadIdx.x == 0) s_bad = (tile_total < 0 || base + tile_total > n_elem) ? 1 : 0;
  for (int e = threadIdx.x; e < n_sb * TILE_P; e += 256) {
    const int b = e / TILE_P, p = e % TILE_P;
    cp[b * (TILE_P + 1) + p] = p < np ? sb_counts[b * npix + p0 + p] : 0u;
  }
  for (int b = threadIdx.x; b < n_sb; b += 256) tp[b] = tile_pos[b * n_tiles + tile];
  __syncthreads();
  // per sub-block: exclusive scan over the tile's pixels (a warp per sub-block)
  for (int b = warp; b < n_sb; b += 8) {
    uint32_t* c = cp + b * (TILE_P + 1);
    const uint32_t a0 = c[lane], a1 = c[32 + lane];
    uint32_t s0 = a0, s1 = a1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y0 = __shfl_up_sync(0xffffffffu, s0, o);
      const uint32_t y1 = __shfl_up_sync(0xffffffffu, s1, o);
      if (lane >= o) {
        s0 += y0;
        s1 += y1;
      }
    }
    const uint32_t t0 = __shfl_sync(0xffffffffu, s0, 31);
    __syncwarp();
    c[lane] = s0 - a0;
    c[32 + lane] = t0 + s1 - a1;
    if (lane == 31) c[TILE_P] = t0 + s1;
  }
  __syncthreads();
  if (threadIdx.x < TILE_P) {
    // per pixel: where its run of each sub-block starts within the tile's lists
    const int p = threadIdx.x;
    if (p < np) {
      int64_t run = static_cast<int64_t>(ev_off[p0 + p]) - base;
      for (int b = 0; b < n_sb; ++b) {
        dst[b * TILE_P + p] = static_cast<uint32_t>(run);
        run += cp[b * (TILE_P + 1) + p + 1] - cp[b * (TILE_P + 1) + p];
      }
      if (run != static_cast<int64_t>(ev_off[p0 + p + 1]) - base) s_bad = 1;
    } else {
      for (int b = 0; b < n_sb; ++b) dst[b * TILE_P + p] = 0;
    }
  } else if (warp == 2) {
    // chunk starts within the walk: exclusive scan of the chunk lengths
    uint32_t carry = 0;
    for (int b0 = 0; b0 < n_sb; b0 += 32) {
      const int b = b0 + lane;
      const uint32_t len = b < n_sb ? cp[b * (TILE_P + 1) + TILE_P] : 0u;
      uint32_t s = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (b < n_sb) cb[b] = carry + s - len;
      carry += __shfl_sync(0xffffffffu, s, 31);
    }
    if (lane == 0) cb[n_sb] = carry;
  }
  __syncthreads();
  const uint32_t total = cb[n_sb];
  if (s_bad || total != tile_total) {
    if (threadIdx.x == 0) atomicOr(err, G2_DEVERR_BOUNDS);
    return;  // block-uniform
  }
  const bool buffered = total <= static_cast<uint32_t>(buf_words);
  uint32_t* out = buffered ? buf : (MODE == GATHER_REL_SPLIT ? reinterpret_cast<uint32_t*>(ev_times) : ev_words) + base;
  bool bad = false;
  if (warp_runs && !(MODE == GATHER_WORDS && sort)) {
    // long runs: a warp takes RUNS consecutive runs at a time (adjacent in the
    // staging area) with its lanes on consecutive words, one load of each run
    // in flight per lane before the stores
    constexpr int RUNS = 4;
    for (int e0 = warp * RUNS; e0 < n_sb * TILE_P; e0 += (256 / 32) * RUNS) {
      uint32_t n[RUNS], d0[RUNS], t_add[RUNS];
      const uint32_t* in[RUNS];
      uint32_t nmax = 0;
#pragma unroll
      for (int r = 0; r < RUNS; ++r) {
        const int e = e0 + r;
        const int b = e / TILE_P, p = e % TILE_P;
        n[r] = 0;
        d0[r] = 0;
        in[r] = stage;
        t_add[r] = MODE == GATHER_REL_WORDS ? static_cast<uint32_t>(b) << 26 : static_cast<uint32_t>(b) * SUBBLOCK;
        if (e >= n_sb * TILE_P || p >= np) continue;
        const uint32_t c0 = cp[b * (TILE_P + 1) + p];
        const uint32_t cnt = cp[b * (TILE_P + 1) + p + 1] - c0;
        const int64_t src = static_cast<int64_t>(tp[b]) + c0;
        const uint32_t d = dst[b * TILE_P + p];
        if (src + cnt > n_elem || static_cast<int64_t>(d) + cnt > total) {
          bad = true;
          continue;
        }
        n[r] = cnt;
        d0[r] = d;
        in[r] = stage + src;
        nmax = cnt > nmax ? cnt : nmax;
      }
      for (uint32_t k = lane; k < nmax; k += 32) {
        uint32_t w[RUNS];
#pragma unroll
        for (int r = 0; r < RUNS; ++r) w[r] = k < n[r] ? in[r][k] : 0u;
#pragma unroll
        for (int r = 0; r < RUNS; ++r) {
          if (k >= n[r]) continue;
          uint32_t* run = out + d0[r];
          if (MODE == GATHER_WORDS) {
            run[k] = w[r];
          } else if (MODE == GATHER_REL_WORDS) {
            run[k] = w[r] + t_add[r];
          } else {
            run[k] = t_add[r] + (w[r] >> 16);  // frame number
            if (buffered)
              bufd[d0[r] + k] = static_cast<uint16_t>(w[r] & 0xFFFFu);
            else
              ev_data[base + d0[r] + k] = static_cast<Tv>(w[r] & 0xFFFFu);
          }
        }
      }
    }
  }
  // a thread per (sub-block, pixel) run (a warp takes 32 consecutive pixels
  // of one sub-block, whose runs are adjacent in the staging area), or, with
  // warp_runs (long runs) and sorting, a warp per run with its lanes on
  // consecutive words
  const int r_first = warp_runs ? ((MODE == GATHER_WORDS && sort) ? (threadIdx.x >> 5) : n_sb * TILE_P)
                                : threadIdx.x;
  const int r_step = warp_runs ? 256 / 32 : 256;
  const uint32_t k0 = warp_runs ? (threadIdx.x & 31) : 0u, k_step = warp_runs ? 32u : 1u;
  for (int e = r_first; e < n_sb * TILE_P; e += r_step) {
    const int b = e / TILE_P, p = e % TILE_P;
    if (p >= np) continue;
    const uint32_t c0 = cp[b * (TILE_P + 1) + p];
    const uint32_t n = cp[b * (TILE_P + 1) + p + 1] - c0;
    if (n == 0) continue;
    const int64_t src = static_cast<int64_t>(tp[b]) + c0;
    const uint32_t d0 = dst[b * TILE_P + p];
    if (src + n > n_elem || static_cast<int64_t>(d0) + n > total) {
      bad = true;
      continue;
    }
    uint32_t* run = out + d0;
    const uint32_t* in = stage + src;
    if (MODE == GATHER_WORDS) {
#pragma unroll 4
      for (uint32_t k = k0; k < n; k += k_step) run[k] = in[k];
    } else if (MODE == GATHER_REL_WORDS) {
      const uint32_t add = static_cast<uint32_t>(b) << 26;  // (b * 1024) << 16
#pragma unroll 4
      for (uint32_t k = k0; k < n; k += k_step) run[k] = in[k] + add;
    } else {
      const uint32_t t_add = static_cast<uint32_t>(b) * SUBBLOCK;
#pragma unroll 4
      for (uint32_t k = k0; k < n; k += k_step) {
        const uint32_t w = in[k];
        run[k] = t_add + (w >> 16);  // frame number
        if (buffered)
          bufd[d0 + k] = static_cast<uint16_t>(w & 0xFFFFu);
        else
          ev_data[base + d0 + k] = static_cast<Tv>(w & 0xFFFFu);
      }
    }
    if (MODE == GATHER_WORDS && sort) {
      if (warp_runs) __syncwarp();
      if (k0 == 0) {
        for (uint32_t m = 1; m < n; ++m) {
          const uint32_t w = run[m];
          uint32_t j = m;
          while (j > 0 && run[j - 1] > w) {
            run[j] = run[j - 1];
            --j;
          }
          run[j] = w;
        }
      }
      if (warp_runs) __syncwarp();
    }
  }
  if (buffered) {
    __syncthreads();
    if (MODE == GATHER_REL_SPLIT) {
      for (uint32_t i = threadIdx.x; i < total; i += 256) {
        ev_times[base + i] = static_cast<int32_t>(buf[i]);
        ev_data[base + i] = static_cast<Tv>(bufd[i]);
      }
    } else {
      for (uint32_t i = threadIdx.x; i < total; i += 256) ev_words[base + i] = buf[i];
    }
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// values[0 .. n] += carry, then carry = values[n] (one block: a running
// exclusive scan continued across calls).
__global__ void __launch_bounds__(1024)
    add_carry_kernel(uint32_t* __restrict__ values, int64_t n, uint32_t* __restrict__ carry) {
  const uint32_t c = *carry;
  __syncthreads();
  for (int64_t i = threadIdx.x; i <= n; i += blockDim.x) values[i] += c;
  __syncthreads();
  if (threadIdx.x == 0) *carry = values[n];
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

extern "C" int g2_add_carry_u32(uint32_t* values_dev, int64_t n, uint32_t* carry_dev, void* stream) {
  using namespace g2;
  if (!values_dev || !carry_dev || n < 0) return G2_ERR_ARG;
  csr::add_carry_kernel<<<1, 1024, 0, as_stream(stream)>>>(values_dev, n, carry_dev);
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
                                    uint16_t* sb_counts_dev, uint32_t* row_totals_dev, int32_t* err_dev,
                                    void* stream) {
  using namespace g2;
  if (!indices_dev || !indptr_dev || !offsets_dev || !row_bounds_dev || !counts_dev || !sb_counts_dev ||
      !row_totals_dev || !err_dev)
    return G2_ERR_ARG;
  if ((index_bytes != 4 && index_bytes != 8) || n_elem < 0 || nframes <= 0 || height <= 0 || width <= 0)
    return G2_ERR_ARG;
  if (width > csr::ROW_MAX_W || height > 65535 || n_elem >= (1ll << 32)) return G2_ERR_UNSUPPORTED;
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
  const int64_t n_sb64 = (static_cast<int64_t>(nframes) + csr::SUBBLOCK - 1) / csr::SUBBLOCK;
  const int64_t smem = (static_cast<int64_t>(width) + 8 * 66) * 4;
  const dim3 grid(static_cast<unsigned>(n_sb64), static_cast<unsigned>(height));
  if (index_bytes == 4) {
    if (!allow_smem(csr::row_count_blocked_kernel<uint32_t>, smem)) return G2_ERR_CUDA;
    csr::row_count_blocked_kernel<uint32_t><<<grid, 256, smem, st>>>(reinterpret_cast<const uint32_t*>(indices_dev),
                                                                     row_bounds_dev, n_elem, nframes, height, width,
                                                                     sb_counts_dev, row_totals_dev, err_dev);
  } else {
    if (!allow_smem(csr::row_count_blocked_kernel<int64_t>, smem)) return G2_ERR_CUDA;
    csr::row_count_blocked_kernel<int64_t><<<grid, 256, smem, st>>>(reinterpret_cast<const int64_t*>(indices_dev),
                                                                    row_bounds_dev, n_elem, nframes, height, width,
                                                                    sb_counts_dev, row_totals_dev, err_dev);
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

namespace {
// Words of the shared-memory buffer of a stage region or a gather tile: a
// little above the mean (uniform data fits), between 1024 and 16384.
// Warp per (sub-block, pixel) run in the gather when runs average 16 words or more.
int warp_runs(int64_t n_elem, int64_t n_sb, int64_t npix) { return n_elem >= 16 * n_sb * npix ? 1 : 0; }

int buffer_words(int64_t n_elem, int64_t units) {
  const int64_t mean = units > 0 ? n_elem / units : n_elem;
  const int64_t w = mean + mean / 16 + 512;
  return static_cast<int>(w < 1024 ? 1024 : (w > 16384 ? 16384 : w));
}
}  // namespace

namespace {
int stage_frames(const void* data_dev, int32_t elem_bytes, const void* indices_dev, const uint32_t* row_bounds_dev,
                 int32_t index_bytes, int64_t n_elem, int32_t frame0, int32_t nframes, int64_t frame_elems,
                 int32_t height, int32_t width, const uint16_t* sb_counts_dev, const uint32_t* row_base_dev,
                 uint32_t* tile_pos_dev, uint32_t* stage_dev, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!data_dev || !indices_dev || !row_bounds_dev || !sb_counts_dev || !row_base_dev || !tile_pos_dev ||
      !stage_dev || !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || (index_bytes != 4 && index_bytes != 8) || n_elem < 0 ||
      nframes <= 0 || height <= 0 || width <= 0 || frame0 < 0 || frame0 % csr::SUBBLOCK != 0 || frame_elems < 0)
    return G2_ERR_ARG;
  if (static_cast<int64_t>(frame0) + nframes > 65536 || width > csr::ROW_MAX_W || height > 65535 ||
      n_elem >= (1ll << 32))
    return G2_ERR_UNSUPPORTED;
  const int64_t n_sb = (static_cast<int64_t>(nframes) + csr::SUBBLOCK - 1) / csr::SUBBLOCK;
  const int64_t npix = static_cast<int64_t>(height) * width;
  const int64_t n_tiles = (npix + csr::TILE_P - 1) / csr::TILE_P;
  const int buf = buffer_words(frame_elems, n_sb * height);
  const int64_t smem = (static_cast<int64_t>(width) + (csr::STAGE_THREADS / 32) * 66 + buf) * 4;
  const dim3 grid(static_cast<unsigned>(n_sb), static_cast<unsigned>(height));
  cudaStream_t st = as_stream(stream);
#define G2_ST(TV, TI)                                                                                              \
  do {                                                                                                             \
    if (!allow_smem(csr::row_stage_kernel<TV, TI>, smem)) return G2_ERR_CUDA;                                      \
    csr::row_stage_kernel<TV, TI><<<grid, csr::STAGE_THREADS, smem, st>>>(                                         \
        reinterpret_cast<const TV*>(data_dev), reinterpret_cast<const TI*>(indices_dev), row_bounds_dev, n_elem,    \
        nframes, height, width, sb_counts_dev, row_base_dev, n_tiles, tile_pos_dev, buf, stage_dev, frame0,        \
        err_dev);                                                                                                  \
  } while (0)
  if (elem_bytes == 1 && index_bytes == 4) G2_ST(uint8_t, uint32_t);
  else if (elem_bytes == 1) G2_ST(uint8_t, int64_t);
  else if (index_bytes == 4) G2_ST(uint16_t, uint32_t);
  else G2_ST(uint16_t, int64_t);
#undef G2_ST
  return launch_status();
}
}  // namespace

extern "C" int g2_csr_stage_blocked(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                                    const uint32_t* row_bounds_dev, int32_t index_bytes, int64_t n_elem,
                                    int32_t nframes, int32_t height, int32_t width, const uint16_t* sb_counts_dev,
                                    const uint32_t* row_base_dev, uint32_t* tile_pos_dev, uint32_t* stage_dev,
                                    int32_t* err_dev, void* stream) {
  return stage_frames(data_dev, elem_bytes, indices_dev, row_bounds_dev, index_bytes, n_elem, 0, nframes, n_elem,
                      height, width, sb_counts_dev, row_base_dev, tile_pos_dev, stage_dev, err_dev, stream);
}

extern "C" int g2_csr_stage_frames(const void* data_dev, int32_t elem_bytes, const void* indices_dev,
                                   const uint32_t* row_bounds_dev, int32_t index_bytes, int64_t n_elem,
                                   int32_t frame0, int32_t nframes, int64_t frame_elems, int32_t height,
                                   int32_t width, const uint16_t* sb_counts_dev, const uint32_t* row_base_dev,
                                   uint32_t* tile_pos_dev, uint32_t* stage_dev, int32_t* err_dev, void* stream) {
  return stage_frames(data_dev, elem_bytes, indices_dev, row_bounds_dev, index_bytes, n_elem, frame0, nframes,
                      frame_elems, height, width, sb_counts_dev, row_base_dev, tile_pos_dev, stage_dev, err_dev,
                      stream);
}

extern "C" int g2_csr_gather_blocked(const uint32_t* stage_dev, const uint32_t* tile_pos_dev,
                                     const uint16_t* sb_counts_dev, int32_t nframes, int64_t npix, int64_t n_elem,
                                     const uint32_t* ev_offsets_dev, int32_t sort, uint32_t* ev_words_dev,
                                     int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!stage_dev || !tile_pos_dev || !sb_counts_dev || !ev_offsets_dev || !ev_words_dev || !err_dev)
    return G2_ERR_ARG;
  if (nframes <= 0 || npix <= 0 || n_elem < 0) return G2_ERR_ARG;
  if (nframes > 65536 || n_elem >= (1ll << 32)) return G2_ERR_UNSUPPORTED;
  const int n_sb = static_cast<int>((static_cast<int64_t>(nframes) + csr::SUBBLOCK - 1) / csr::SUBBLOCK);
  const int64_t n_tiles = (npix + csr::TILE_P - 1) / csr::TILE_P;
  if (n_tiles > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int wr = warp_runs(n_elem, n_sb, npix);
  const int buf = wr ? 0 : buffer_words(n_elem * csr::TILE_P, npix);
  const int64_t smem = (131ll * n_sb + 1 + buf) * 4;
  auto kernel = csr::gather_tiles_kernel<csr::GATHER_WORDS, uint8_t>;
  if (!allow_smem(kernel, smem)) return G2_ERR_CUDA;
  kernel<<<static_cast<unsigned>(n_tiles), 256, smem, as_stream(stream)>>>(
      stage_dev, tile_pos_dev, sb_counts_dev, n_sb, npix, n_tiles, ev_offsets_dev, n_elem, sort ? 1 : 0, buf, wr,
      ev_words_dev, nullptr, nullptr, err_dev);
  return launch_status();
}

extern "C" int g2_events_gather_rel(const uint32_t* stage_dev, const uint32_t* tile_pos_dev,
                                    const uint16_t* sb_counts_dev, int32_t nframes, int64_t npix, int64_t n_elem,
                                    const uint32_t* ev_offsets_dev, int32_t elem_bytes, uint32_t* ev_words_dev,
                                    int32_t* ev_times_dev, void* ev_data_dev, int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!stage_dev || !tile_pos_dev || !sb_counts_dev || !ev_offsets_dev || !err_dev) return G2_ERR_ARG;
  if (nframes <= 0 || npix <= 0 || n_elem < 0) return G2_ERR_ARG;
  const bool words = ev_words_dev != nullptr;
  if (words == (ev_times_dev != nullptr || ev_data_dev != nullptr)) return G2_ERR_ARG;  // one output form
  if (!words && (!ev_times_dev || !ev_data_dev || (elem_bytes != 1 && elem_bytes != 2))) return G2_ERR_ARG;
  if (words && nframes > 65536) return G2_ERR_UNSUPPORTED;
  if (n_elem >= (1ll << 32)) return G2_ERR_UNSUPPORTED;
  const int64_t n_sb64 = (static_cast<int64_t>(nframes) + csr::SUBBLOCK - 1) / csr::SUBBLOCK;
  if (n_sb64 > 400) return G2_ERR_TOO_LARGE;  // the tile tables (131 words per sub-block) stay in shared memory
  const int n_sb = static_cast<int>(n_sb64);
  const int64_t n_tiles = (npix + csr::TILE_P - 1) / csr::TILE_P;
  if (n_tiles > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int64_t tables = (131ll * n_sb + 1) * 4, per_word = words ? 4 : 6;
  const int wr = warp_runs(n_elem, n_sb, npix);
  // long runs are copied by whole warps (coalesced): no tile buffer, more CTAs per SM
  int64_t buf = wr ? 0 : buffer_words(n_elem * csr::TILE_P, npix);
  if (tables + buf * per_word > 227 * 1024) buf = (227 * 1024 - tables) / per_word;  // larger tiles go in place
  const int64_t smem = tables + buf * per_word;
  cudaStream_t st = as_stream(stream);
  const unsigned grid = static_cast<unsigned>(n_tiles);
  if (words) {
    auto kernel = csr::gather_tiles_kernel<csr::GATHER_REL_WORDS, uint8_t>;
    if (!allow_smem(kernel, smem)) return G2_ERR_CUDA;
    kernel<<<grid, 256, smem, st>>>(stage_dev, tile_pos_dev, sb_counts_dev, n_sb, npix, n_tiles, ev_offsets_dev,
                                    n_elem, 0, static_cast<int>(buf), wr, ev_words_dev, nullptr, nullptr, err_dev);
  } else if (elem_bytes == 1) {
    auto kernel = csr::gather_tiles_kernel<csr::GATHER_REL_SPLIT, uint8_t>;
    if (!allow_smem(kernel, smem)) return G2_ERR_CUDA;
    kernel<<<grid, 256, smem, st>>>(stage_dev, tile_pos_dev, sb_counts_dev, n_sb, npix, n_tiles, ev_offsets_dev,
                                    n_elem, 0, static_cast<int>(buf), wr, nullptr, ev_times_dev,
                                    reinterpret_cast<uint8_t*>(ev_data_dev),
                                    err_dev);
  } else {
    auto kernel = csr::gather_tiles_kernel<csr::GATHER_REL_SPLIT, uint16_t>;
    if (!allow_smem(kernel, smem)) return G2_ERR_CUDA;
    kernel<<<grid, 256, smem, st>>>(stage_dev, tile_pos_dev, sb_counts_dev, n_sb, npix, n_tiles, ev_offsets_dev,
                                    n_elem, 0, static_cast<int>(buf), wr, nullptr, ev_times_dev,
                                    reinterpret_cast<uint16_t*>(ev_data_dev),
                                    err_dev);
  }
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
