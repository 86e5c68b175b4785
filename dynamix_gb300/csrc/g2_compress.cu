// Frame compression on the device: dense frames -> per-pixel event lists, the
// layout of dynamix's FramesCompressor (correlator/event.py:207-321) that the
// event correlator consumes, with the hot-pixel threshold, sticky mask and sum
// frame of the streaming reader (io/readdata.py:441-468, neigercompress).
//
// Whole stack (compress_all_stack, event.py:267-284), frames (T, H*W):
//   1. count  : one CTA per (1024-frame sub-block, 1024-pixel block), a thread
//               per 4 consecutive pixels; per (sub-block, pixel) the number of
//               positive values (uint16) and, with a threshold, the first
//               frame above it and the positives before that frame;
//   2. finish : per pixel, the sticky mask (input mask, or the first frame
//               above the threshold: that frame and every later one drop out),
//               corrected sub-block counts, the pixel's total, the cut frame;
//   3. scans  : pixel totals -> event offsets; block totals -> block bases;
//   4. stage  : the same CTAs read their frames again and write every kept
//               value as one word ((t - sub-block start) << 16) | v into the
//               staging area, ordered by sub-block, then pixel, then frame;
//   5. gather : the tiled gather of the CSR path (g2_csr.cu) copies the runs
//               into the per-pixel lists and restores absolute frame numbers.
// Values are u8/u16 or i8/i16 (only values > 0 are events, as in the
// reference's `frames > 0`); frame numbers are not limited to 16 bits.
//
// Streaming (process_frame, event.py:286-296): a thread per pixel appends a
// batch of frames' positive values to the (pixels x max_nnz) event and time
// arrays; compaction (get_compacted_events, event.py:298-321) copies each
// pixel's row to its offset.
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace cmp {

constexpr int SUBBLOCK = 1024;       // frames of one sub-block (as in the CSR path)
constexpr int PX = 4;                // consecutive pixels of one thread
constexpr int THREADS = 256;
constexpr int BLK_PX = THREADS * PX;  // pixels of one CTA
constexpr int TILE_P = 64;           // pixels of one gather tile (as in the CSR path)
constexpr int STAGE_BUF = 16384;     // words of a CTA region assembled in shared memory (dynamic, 64 KB)
constexpr int WCAP = STAGE_BUF / (2 * (THREADS / 32));  // words of one warp's chunk (words + positions)
constexpr uint16_t NONE = 0xFFFFu;

// Four consecutive values of one frame as int32 (sign-extended for signed
// types).  VEC: one 4- or 8-byte load (the frame stride and the base allow it).
template <typename Tv, bool VEC>
__device__ __forceinline__ void load4(const Tv* __restrict__ src, int64_t n_valid, int32_t v[PX]) {
  if (VEC) {
    if (sizeof(Tv) == 1) {
      const uint32_t w = *reinterpret_cast<const uint32_t*>(src);
#pragma unroll
      for (int j = 0; j < PX; ++j) {
        const uint32_t b = (w >> (8 * j)) & 0xFFu;
        v[j] = static_cast<Tv>(-1) < 0 ? static_cast<int32_t>(static_cast<int8_t>(b)) : static_cast<int32_t>(b);
      }
    } else {
      const uint2 w = *reinterpret_cast<const uint2*>(src);
      const uint32_t h[PX] = {w.x & 0xFFFFu, w.x >> 16, w.y & 0xFFFFu, w.y >> 16};
#pragma unroll
      for (int j = 0; j < PX; ++j)
        v[j] = static_cast<Tv>(-1) < 0 ? static_cast<int32_t>(static_cast<int16_t>(h[j]))
                                       : static_cast<int32_t>(h[j]);
    }
  } else {
#pragma unroll
    for (int j = 0; j < PX; ++j) v[j] = j < n_valid ? static_cast<int32_t>(src[j]) : 0;
  }
}

// Raw word holding 4 consecutive values (VEC loads) and its unpacking.
template <typename Tv> struct Word4 { using type = uint32_t; };
template <> struct Word4<uint16_t> { using type = uint2; };
template <> struct Word4<int16_t> { using type = uint2; };

template <typename Tv>
__device__ __forceinline__ void unpack4(uint32_t w, int32_t v[PX]) {
#pragma unroll
  for (int j = 0; j < PX; ++j) {
    const uint32_t b = (w >> (8 * j)) & 0xFFu;
    v[j] = static_cast<Tv>(-1) < 0 ? static_cast<int32_t>(static_cast<int8_t>(b)) : static_cast<int32_t>(b);
  }
}
template <typename Tv>
__device__ __forceinline__ void unpack4(uint2 w, int32_t v[PX]) {
  const uint32_t h[PX] = {w.x & 0xFFFFu, w.x >> 16, w.y & 0xFFFFu, w.y >> 16};
#pragma unroll
  for (int j = 0; j < PX; ++j)
    v[j] = static_cast<Tv>(-1) < 0 ? static_cast<int32_t>(static_cast<int16_t>(h[j])) : static_cast<int32_t>(h[j]);
}

// Value j of the 4 in a raw word.
template <typename Tv>
__device__ __forceinline__ int32_t lane_value(uint32_t w, int j) {
  const uint32_t b = (w >> (8 * j)) & 0xFFu;
  return static_cast<Tv>(-1) < 0 ? static_cast<int32_t>(static_cast<int8_t>(b)) : static_cast<int32_t>(b);
}
template <typename Tv>
__device__ __forceinline__ int32_t lane_value(uint2 w, int j) {
  const uint32_t h = ((j < 2 ? w.x : w.y) >> (16 * (j & 1))) & 0xFFFFu;
  return static_cast<Tv>(-1) < 0 ? static_cast<int32_t>(static_cast<int16_t>(h)) : static_cast<int32_t>(h);
}

// Positive-value flags of a 32-bit word of packed values, all lanes at once:
// the top bit of each 8-bit (u8/i8) or 16-bit (u16/i16) lane is set when the
// lane's value is > 0.  Adding the low bits to all-ones-but-top carries into
// the top bit when any low bit is set (never across lanes); unsigned values
// are positive when any bit is set, signed ones when in addition the sign bit
// is clear.
template <typename Tv>
__device__ __forceinline__ uint32_t positive_flags(uint32_t w) {
  constexpr uint32_t low = sizeof(Tv) == 1 ? 0x7F7F7F7Fu : 0x7FFF7FFFu;
  const uint32_t any_low = (w & low) + low;
  return (static_cast<Tv>(-1) < 0 ? (any_low & ~w) : (any_low | w)) & ~low;
}

// Lane counters of positive values: a0 holds 4 byte counters (8-bit values,
// at most 255 frames between flushes) or, with a1, 4 16-bit counters.
template <typename Tv>
__device__ __forceinline__ void add_positive(uint32_t w, uint32_t& a0, uint32_t&) {
  a0 += positive_flags<Tv>(w) >> 7;
}
template <typename Tv>
__device__ __forceinline__ void add_positive(uint2 w, uint32_t& a0, uint32_t& a1) {
  a0 += positive_flags<Tv>(w.x) >> 15;
  a1 += positive_flags<Tv>(w.y) >> 15;
}
template <typename Tv>
__device__ __forceinline__ void flush_positive(uint32_t& a0, uint32_t& a1, uint32_t c[PX]) {
  if (sizeof(Tv) == 1) {
#pragma unroll
    for (int j = 0; j < PX; ++j) c[j] += (a0 >> (8 * j)) & 0xFFu;
  } else {
    c[0] += a0 & 0xFFFFu;
    c[1] += a0 >> 16;
    c[2] += a1 & 0xFFFFu;
    c[3] += a1 >> 16;
  }
  a0 = 0;
  a1 = 0;
}

// frames whose loads are in flight together (VEC): 64 bytes per thread
template <typename Tv> struct InFlight { static constexpr int frames = sizeof(Tv) == 1 ? 16 : 8; };

// Walk frames [t, t1) of 4 pixels at src (frame stride npix), calling
// f(v, t) per frame: with VEC, 64 bytes of loads per thread are issued
// before they are used.
// `more()` may stop the walk between groups of frames.
template <typename Tv, bool VEC, typename F, typename M>
__device__ __forceinline__ void walk_frames(const Tv* __restrict__ src, int64_t npix, int64_t t, int64_t t1,
                                            int64_t n_valid, F&& f, M&& more) {
  if (VEC) {
    using W = typename Word4<Tv>::type;
    constexpr int TU = InFlight<Tv>::frames;
    for (; t + TU <= t1 && more(); t += TU) {
      W raw[TU];
#pragma unroll
      for (int u = 0; u < TU; ++u) raw[u] = *reinterpret_cast<const W*>(src + u * npix);
#pragma unroll
      for (int u = 0; u < TU; ++u) {
        int32_t v[PX];
        unpack4<Tv>(raw[u], v);
        f(v, t + u);
      }
      src += TU * npix;
    }
  }
  for (; t + 4 <= t1 && more(); t += 4) {
    int32_t v[4][PX];
#pragma unroll
    for (int u = 0; u < 4; ++u) load4<Tv, VEC>(src + u * npix, n_valid, v[u]);
#pragma unroll
    for (int u = 0; u < 4; ++u) f(v[u], t + u);
    src += 4 * npix;
  }
  for (; t < t1 && more(); ++t) {
    int32_t v[PX];
    load4<Tv, VEC>(src, n_valid, v);
    f(v, t);
    src += npix;
  }
}

// Positive values of frames [0, n) of 4 pixels at src (VEC loads), added to
// cnt: lane counters flushed every 128 frames.
template <typename Tv>
__device__ __forceinline__ void count_positive(const Tv* __restrict__ src, int64_t npix, int64_t n,
                                               uint32_t cnt[PX]) {
  using W = typename Word4<Tv>::type;
  constexpr int TU = InFlight<Tv>::frames;
  uint32_t a0 = 0, a1 = 0;
  int64_t t = 0;
  for (int g = 1; t + TU <= n; t += TU, ++g) {
    W raw[TU];
#pragma unroll
    for (int u = 0; u < TU; ++u) raw[u] = *reinterpret_cast<const W*>(src + (t + u) * npix);
#pragma unroll
    for (int u = 0; u < TU; ++u) add_positive<Tv>(raw[u], a0, a1);
    if (g % (128 / TU) == 0) flush_positive<Tv>(a0, a1, cnt);
  }
  for (; t < n; ++t) add_positive<Tv>(*reinterpret_cast<const W*>(src + t * npix), a0, a1);
  flush_positive<Tv>(a0, a1, cnt);
}

// Block-wide exclusive scan of one uint32 per thread; returns the prefix and
// the block total.  s_warp: [THREADS / 32] shared words.
__device__ __forceinline__ uint32_t block_scan(uint32_t x, uint32_t* s_warp, uint32_t& total) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) s_warp[warp] = inc;
  __syncthreads();
  uint32_t before = 0, all = 0;
#pragma unroll
  for (int w = 0; w < THREADS / 32; ++w) {
    const uint32_t s = s_warp[w];
    before += w < warp ? s : 0u;
    all += s;
  }
  __syncthreads();  // s_warp may be reused
  total = all;
  return before + inc - x;
}

// Pass 1.  sb_first / sb_before are written only with THR, sum_frame only
// with SUM.
template <typename Tv, bool VEC, bool THR, bool SUM>
__global__ void __launch_bounds__(THREADS)
    count_kernel(const Tv* __restrict__ frames, int32_t T, int64_t npix, int32_t thr,
                 uint16_t* __restrict__ sb_counts, uint16_t* __restrict__ sb_first, uint16_t* __restrict__ sb_before,
                 uint32_t* __restrict__ blk_totals, long long* __restrict__ sum_frame) {
  __shared__ uint32_t s_warp[THREADS / 32];
  const int64_t sb = blockIdx.x;
  const int64_t n_blk = gridDim.y;
  const int64_t p0 = static_cast<int64_t>(blockIdx.y) * BLK_PX + static_cast<int64_t>(threadIdx.x) * PX;
  const int64_t n_valid = p0 < npix ? (npix - p0 < PX ? npix - p0 : PX) : 0;
  const int64_t t0 = sb * SUBBLOCK;
  const int64_t t1 = t0 + SUBBLOCK < T ? t0 + SUBBLOCK : T;
  uint32_t cnt[PX] = {0, 0, 0, 0};
  uint32_t before[PX] = {0, 0, 0, 0};
  uint32_t first[PX] = {NONE, NONE, NONE, NONE};
  long long sum[PX] = {0, 0, 0, 0};
  if (n_valid > 0) {
    if (VEC && !THR && !SUM) {
      count_positive<Tv>(frames + t0 * npix + p0, npix, t1 - t0, cnt);
    } else {
      walk_frames<Tv, VEC>(
          frames + t0 * npix + p0, npix, t0, t1, n_valid,
          [&](const int32_t v[PX], int64_t t) {
#pragma unroll
            for (int j = 0; j < PX; ++j) {
              if (THR && v[j] > thr && first[j] == NONE) {
                first[j] = static_cast<uint32_t>(t - t0);
                before[j] = cnt[j];
              }
              cnt[j] += v[j] > 0 ? 1u : 0u;
              if (SUM) sum[j] += v[j];
            }
          },
          [] { return true; });
    }
#pragma unroll
    for (int j = 0; j < PX; ++j) {
      if (j >= n_valid) break;
      const int64_t p = p0 + j;
      sb_counts[sb * npix + p] = static_cast<uint16_t>(cnt[j]);  // <= SUBBLOCK
      if (THR) {
        sb_first[sb * npix + p] = static_cast<uint16_t>(first[j]);
        sb_before[sb * npix + p] = static_cast<uint16_t>(before[j]);
      }
      if (SUM && sum[j] != 0)
        atomicAdd(reinterpret_cast<unsigned long long*>(&sum_frame[p]), static_cast<unsigned long long>(sum[j]));
    }
  }
  uint32_t total;
  block_scan(cnt[0] + cnt[1] + cnt[2] + cnt[3], s_warp, total);
  if (threadIdx.x == 0) blk_totals[sb * n_blk + blockIdx.y] = total;
}

// Pass 2: the sticky mask.  Per pixel, in sub-block order: a masked pixel
// keeps nothing; otherwise the first sub-block holding a value above the
// threshold keeps only the positives before it, and later sub-blocks nothing.
// The removed counts come off the block totals.  Also the pixel's total, the
// cut frame (T when nothing is cut) and the mask after the stack.
template <bool THR>
__global__ void __launch_bounds__(THREADS)
    finish_kernel(uint16_t* __restrict__ sb_counts, const uint16_t* __restrict__ sb_first,
                  const uint16_t* __restrict__ sb_before, int n_sb, int32_t T, int64_t npix,
                  uint8_t* __restrict__ mask, uint32_t* __restrict__ blk_totals, int64_t n_blk,
                  uint32_t* __restrict__ counts, int32_t* __restrict__ t_cut) {
  for (int64_t p = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; p < npix;
       p += static_cast<int64_t>(gridDim.x) * THREADS) {
    const bool masked = mask != nullptr && mask[p] != 0;
    int64_t cut = masked ? 0 : T;
    uint32_t total = 0;
    const int64_t blk = p / BLK_PX;
    for (int b = 0; b < n_sb; ++b) {
      const int64_t i = static_cast<int64_t>(b) * npix + p;
      const uint32_t c = sb_counts[i];
      uint32_t keep = c;
      if (static_cast<int64_t>(b) * SUBBLOCK >= cut) {
        keep = 0;
      } else if (THR && sb_first[i] != NONE) {
        keep = sb_before[i];
        cut = static_cast<int64_t>(b) * SUBBLOCK + sb_first[i];
      }
      if (keep != c) {
        sb_counts[i] = static_cast<uint16_t>(keep);
        atomicSub(&blk_totals[static_cast<int64_t>(b) * n_blk + blk], c - keep);
      }
      total += keep;
    }
    counts[p] = total;
    if (t_cut) t_cut[p] = static_cast<int32_t>(cut);
    if (mask) mask[p] = cut < T ? 1 : 0;
  }
}

// Pass 4 (after the scans).  A thread's 4 pixels get their run starts from a
// block scan of the sub-block counts; the region of the CTA is assembled in
// shared memory when it fits (coalesced write-out), else each warp assembles
// chunks of frames in its shared slice (coalesced within each pixel's piece).
template <typename Tv, bool VEC, bool CUT>
__global__ void __launch_bounds__(THREADS)
    stage_kernel(const Tv* __restrict__ frames, int32_t T, int64_t npix, const uint16_t* __restrict__ sb_counts,
                 const int32_t* __restrict__ t_cut, const uint32_t* __restrict__ blk_base, int64_t n_tiles,
                 uint32_t* __restrict__ tile_pos, uint32_t* __restrict__ stage, int64_t n_stage,
                 int32_t* __restrict__ err) {
  __shared__ uint32_t s_warp[THREADS / 32];
  extern __shared__ uint32_t buf[];  // STAGE_BUF words
  const int64_t sb = blockIdx.x;
  const int64_t n_blk = gridDim.y;
  const int64_t p0 = static_cast<int64_t>(blockIdx.y) * BLK_PX + static_cast<int64_t>(threadIdx.x) * PX;
  const int64_t n_valid = p0 < npix ? (npix - p0 < PX ? npix - p0 : PX) : 0;
  const int64_t t0 = sb * SUBBLOCK;
  const int64_t t1 = t0 + SUBBLOCK < T ? t0 + SUBBLOCK : T;
  uint32_t c[PX];
  int64_t cut[PX];
#pragma unroll
  for (int j = 0; j < PX; ++j) {
    c[j] = j < n_valid ? sb_counts[sb * npix + p0 + j] : 0u;
    cut[j] = CUT && j < n_valid ? static_cast<int64_t>(t_cut[p0 + j]) : static_cast<int64_t>(T);
  }
  uint32_t total;
  const uint32_t own = c[0] + c[1] + c[2] + c[3];
  const uint32_t prefix = block_scan(own, s_warp, total);
  const int64_t base = blk_base[sb * n_blk + blockIdx.y];
  const bool skip = base + total > n_stage;  // block-uniform
  const bool buffered = total <= static_cast<uint32_t>(STAGE_BUF);
  uint32_t cur[PX], end[PX];
  uint32_t run = prefix;
#pragma unroll
  for (int j = 0; j < PX; ++j) {
    cur[j] = run;
    run += c[j];
    end[j] = run;
    const int64_t p = p0 + j;
    if (j < n_valid && p % TILE_P == 0) tile_pos[sb * n_tiles + p / TILE_P] = static_cast<uint32_t>(base + cur[j]);
  }
  bool bad = skip;
  const uint32_t goal = end[0] + end[1] + end[2] + end[3];
  int64_t t = t0;
  if (VEC && !skip && !buffered) {
    // Region too large for shared memory: each warp takes CHUNK frames of its
    // 128 pixels at a time, counts them from registers, scans the counts
    // across the warp and assembles the chunk's words pixel-major in its own
    // shared slice, then writes them out with consecutive lanes on
    // consecutive words (each pixel's words of the chunk are one contiguous
    // piece of its run).  A chunk with more than WCAP words, or with more
    // values than a pixel's run has room for, is written word by word.
    using W = typename Word4<Tv>::type;
    constexpr int CHUNK = 2 * InFlight<Tv>::frames;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t* wb = buf + (threadIdx.x >> 5) * (2 * WCAP);
    uint32_t* wd = wb + WCAP;
    const Tv* src = frames + t0 * npix + p0;
    for (; t + CHUNK <= t1; t += CHUNK, src += CHUNK * npix) {
      const bool mine = own > 0 && cur[0] + cur[1] + cur[2] + cur[3] < goal;
      if (!__any_sync(0xffffffffu, mine)) break;
      W raw[CHUNK];
#pragma unroll
      for (int u = 0; u < CHUNK; ++u) raw[u] = mine ? *reinterpret_cast<const W*>(src + u * npix) : W{};
      uint32_t c[PX] = {0u, 0u, 0u, 0u};
      if (CUT) {
#pragma unroll
        for (int u = 0; u < CHUNK; ++u) {
          int32_t v[PX];
          unpack4<Tv>(raw[u], v);
#pragma unroll
          for (int j = 0; j < PX; ++j) c[j] += v[j] > 0 && t + u < cut[j] ? 1u : 0u;
        }
      } else {
        uint32_t a0 = 0, a1 = 0;  // CHUNK < 256 frames: no flush before the end
#pragma unroll
        for (int u = 0; u < CHUNK; ++u) add_positive<Tv>(raw[u], a0, a1);
        flush_positive<Tv>(a0, a1, c);
      }
      bool over = false;
#pragma unroll
      for (int j = 0; j < PX; ++j) over |= cur[j] + c[j] > end[j];
      const uint32_t n = c[0] + c[1] + c[2] + c[3];
      uint32_t incl = n;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= static_cast<uint32_t>(o)) incl += y;
      }
      const uint32_t wtotal = __shfl_sync(0xffffffffu, incl, 31);
      const uint32_t rel0 = static_cast<uint32_t>(t - t0);
      if (__any_sync(0xffffffffu, over) || wtotal > static_cast<uint32_t>(WCAP)) {
#pragma unroll
        for (int u = 0; u < CHUNK; ++u) {
          int32_t v[PX];
          unpack4<Tv>(raw[u], v);
#pragma unroll
          for (int j = 0; j < PX; ++j) {
            if (v[j] > 0 && (!CUT || t + u < cut[j])) {
              if (cur[j] < end[j]) {
                stage[base + cur[j]] = ((rel0 + u) << 16) | (static_cast<uint32_t>(v[j]) & 0xFFFFu);
                ++cur[j];
              } else {
                bad = true;
              }
            }
          }
        }
      } else {
        uint32_t pos = incl - n;
#pragma unroll
        for (int j = 0; j < PX; ++j) {
#pragma unroll
          for (int u = 0; u < CHUNK; ++u) {
            const int32_t v = lane_value<Tv>(raw[u], j);
            if (v > 0 && (!CUT || t + u < cut[j])) {
              wb[pos] = ((rel0 + u) << 16) | (static_cast<uint32_t>(v) & 0xFFFFu);
              wd[pos] = cur[j];
              ++pos;
              ++cur[j];
            }
          }
        }
        __syncwarp();
        for (uint32_t i = lane; i < wtotal; i += 32) stage[base + wd[i]] = wb[i];
        __syncwarp();
      }
    }
  }
  if (!skip && own > 0 && t < t1) {
    walk_frames<Tv, VEC>(
        frames + t * npix + p0, npix, t, t1, n_valid,
        [&](const int32_t v[PX], int64_t tf) {
          const uint32_t rel = static_cast<uint32_t>(tf - t0);
#pragma unroll
          for (int j = 0; j < PX; ++j) {
            if (v[j] > 0 && tf < cut[j]) {
              if (cur[j] < end[j]) {
                const uint32_t w = (rel << 16) | (static_cast<uint32_t>(v[j]) & 0xFFFFu);
                if (buffered)
                  buf[cur[j]] = w;
                else
                  stage[base + cur[j]] = w;
                ++cur[j];
              } else {
                bad = true;
              }
            }
          }
        },
        [&] { return cur[0] + cur[1] + cur[2] + cur[3] < goal; });  // every event placed: stop reading
  }
  if (buffered && !skip) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < total; i += THREADS) stage[base + i] = buf[i];
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Streaming: a thread per pixel appends the positive values of nb frames
// (frame numbers frame0, frame0 + 1, ...) to its row of the (npix x max_nnz)
// event and time arrays.  With a threshold, a value above it masks the pixel
// from that frame on (the mask persists across calls); sum_frame adds the raw
// values (before masking).  A pixel past max_nnz events keeps max_nnz and
// sets G2_DEVERR_RANGE.
template <typename Tv, bool THR>
__global__ void __launch_bounds__(THREADS)
    stream_kernel(const Tv* __restrict__ frames, int32_t nb, int64_t frame0, int64_t npix, int32_t max_nnz,
                  int32_t thr, uint8_t* __restrict__ mask, long long* __restrict__ sum_frame,
                  Tv* __restrict__ events, int32_t* __restrict__ times, int32_t* __restrict__ counter,
                  int32_t* __restrict__ err) {
  bool over = false;
  for (int64_t p = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; p < npix;
       p += static_cast<int64_t>(gridDim.x) * THREADS) {
    int32_t c = counter[p];
    if (c < 0 || c > max_nnz) {
      over = true;
      c = c < 0 ? 0 : max_nnz;
    }
    bool m = mask != nullptr && mask[p] != 0;
    long long s = 0;
    for (int32_t b = 0; b < nb; ++b) {
      int32_t v = static_cast<int32_t>(frames[static_cast<int64_t>(b) * npix + p]);
      s += v;
      if (THR && v > thr) m = true;
      if (m) v = 0;
      if (v > 0) {
        if (c < max_nnz) {
          events[p * max_nnz + c] = static_cast<Tv>(v);
          times[p * max_nnz + c] = static_cast<int32_t>(frame0 + b);
          ++c;
        } else {
          over = true;
        }
      }
    }
    counter[p] = c;
    if (mask) mask[p] = m ? 1 : 0;
    if (sum_frame) sum_frame[p] += s;
  }
  if (over) atomicOr(err, G2_DEVERR_RANGE);
}

// Streaming compaction: pixel p's counter[p] events go to offsets[p] ...
template <typename Tv>
__global__ void __launch_bounds__(THREADS)
    compact_kernel(const Tv* __restrict__ events, const int32_t* __restrict__ times,
                   const int32_t* __restrict__ counter, int64_t npix, int32_t max_nnz,
                   const uint32_t* __restrict__ offsets, int64_t cap, Tv* __restrict__ out_data,
                   int32_t* __restrict__ out_times, int32_t* __restrict__ err) {
  bool bad = false;
  for (int64_t p = blockIdx.x * static_cast<int64_t>(THREADS) + threadIdx.x; p < npix;
       p += static_cast<int64_t>(gridDim.x) * THREADS) {
    const int32_t n = counter[p];
    const int64_t o = offsets[p];
    if (n < 0 || n > max_nnz || o + n > cap || o + n != static_cast<int64_t>(offsets[p + 1])) {
      bad = true;
      continue;
    }
    for (int32_t k = 0; k < n; ++k) {
      out_data[o + k] = events[p * max_nnz + k];
      out_times[o + k] = times[p * max_nnz + k];
    }
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

}  // namespace cmp
}  // namespace g2

namespace {
using namespace g2;

int n_blocks(int64_t n, int64_t per, int sms, int waves) {
  int64_t b = (n + per - 1) / per;
  const int64_t cap = static_cast<int64_t>(sms) * waves;
  return static_cast<int>(b < 1 ? 1 : (b > cap ? cap : b));
}

bool kind_ok(int32_t k) { return k == 1 || k == 2 || k == -1 || k == -2; }
int64_t kind_bytes(int32_t k) { return k < 0 ? -k : k; }

template <typename Tv, bool SUM>
void launch_count_sum(const Tv* f, bool vec, bool thr_on, dim3 grid, cudaStream_t st, int32_t T, int64_t npix,
                      int32_t thr, uint16_t* sbc, uint16_t* sbf, uint16_t* sbb, uint32_t* blk, long long* sum) {
  if (vec && thr_on)
    cmp::count_kernel<Tv, true, true, SUM><<<grid, cmp::THREADS, 0, st>>>(f, T, npix, thr, sbc, sbf, sbb, blk, sum);
  else if (vec)
    cmp::count_kernel<Tv, true, false, SUM><<<grid, cmp::THREADS, 0, st>>>(f, T, npix, thr, sbc, sbf, sbb, blk, sum);
  else if (thr_on)
    cmp::count_kernel<Tv, false, true, SUM><<<grid, cmp::THREADS, 0, st>>>(f, T, npix, thr, sbc, sbf, sbb, blk, sum);
  else
    cmp::count_kernel<Tv, false, false, SUM><<<grid, cmp::THREADS, 0, st>>>(f, T, npix, thr, sbc, sbf, sbb, blk,
                                                                           sum);
}

template <typename Tv>
void launch_count(const void* frames, bool vec, bool thr_on, dim3 grid, cudaStream_t st, int32_t T, int64_t npix,
                  int32_t thr, uint16_t* sbc, uint16_t* sbf, uint16_t* sbb, uint32_t* blk, long long* sum) {
  const Tv* f = reinterpret_cast<const Tv*>(frames);
  if (sum)
    launch_count_sum<Tv, true>(f, vec, thr_on, grid, st, T, npix, thr, sbc, sbf, sbb, blk, sum);
  else
    launch_count_sum<Tv, false>(f, vec, thr_on, grid, st, T, npix, thr, sbc, sbf, sbb, blk, sum);
}

template <typename Tv, bool VEC, bool CUT>
int launch_stage_as(const Tv* f, dim3 grid, cudaStream_t st, int32_t T, int64_t npix, const uint16_t* sbc,
                    const int32_t* cut, const uint32_t* base, int64_t n_tiles, uint32_t* tpos, uint32_t* stage,
                    int64_t n_stage, int32_t* err) {
  constexpr int smem = cmp::STAGE_BUF * 4;
  if (cudaFuncSetAttribute(cmp::stage_kernel<Tv, VEC, CUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) !=
      cudaSuccess)
    return G2_ERR_CUDA;
  cmp::stage_kernel<Tv, VEC, CUT><<<grid, cmp::THREADS, smem, st>>>(f, T, npix, sbc, cut, base, n_tiles, tpos, stage,
                                                                    n_stage, err);
  return G2_OK;
}

template <typename Tv>
int launch_stage(const void* frames, bool vec, bool cut_on, dim3 grid, cudaStream_t st, int32_t T, int64_t npix,
                 const uint16_t* sbc, const int32_t* cut, const uint32_t* base, int64_t n_tiles, uint32_t* tpos,
                 uint32_t* stage, int64_t n_stage, int32_t* err) {
  const Tv* f = reinterpret_cast<const Tv*>(frames);
  if (vec && cut_on)
    return launch_stage_as<Tv, true, true>(f, grid, st, T, npix, sbc, cut, base, n_tiles, tpos, stage, n_stage, err);
  if (vec)
    return launch_stage_as<Tv, true, false>(f, grid, st, T, npix, sbc, cut, base, n_tiles, tpos, stage, n_stage, err);
  if (cut_on)
    return launch_stage_as<Tv, false, true>(f, grid, st, T, npix, sbc, cut, base, n_tiles, tpos, stage, n_stage, err);
  return launch_stage_as<Tv, false, false>(f, grid, st, T, npix, sbc, cut, base, n_tiles, tpos, stage, n_stage, err);
}

// Grid of the count and stage passes: (sub-blocks, 1024-pixel blocks).
int stack_grid(int32_t nframes, int64_t npix, dim3& grid) {
  const int64_t n_sb = (static_cast<int64_t>(nframes) + cmp::SUBBLOCK - 1) / cmp::SUBBLOCK;
  const int64_t n_blk = (npix + cmp::BLK_PX - 1) / cmp::BLK_PX;
  if (n_blk > 65535 || n_sb > 0x7fffffff) return G2_ERR_TOO_LARGE;
  grid = dim3(static_cast<unsigned>(n_sb), static_cast<unsigned>(n_blk));
  return G2_OK;
}
}  // namespace

extern "C" int g2_compress_count(const void* frames_dev, int32_t elem_kind, int32_t nframes, int64_t npix,
                                 int32_t threshold, uint16_t* sb_counts_dev, uint16_t* sb_first_dev,
                                 uint16_t* sb_before_dev, uint32_t* blk_totals_dev, int64_t* sum_frame_dev,
                                 void* stream) {
  if (!frames_dev || !sb_counts_dev || !blk_totals_dev || !kind_ok(elem_kind) || nframes <= 0 || npix <= 0)
    return G2_ERR_ARG;
  const bool thr_on = threshold >= 0;
  if (thr_on && (!sb_first_dev || !sb_before_dev)) return G2_ERR_ARG;
  dim3 grid;
  const int rc = stack_grid(nframes, npix, grid);
  if (rc != G2_OK) return rc;
  const int64_t eb = kind_bytes(elem_kind);
  const bool vec = npix % cmp::PX == 0 && aligned(frames_dev, static_cast<uintptr_t>(eb * cmp::PX));
  cudaStream_t st = as_stream(stream);
  long long* sum = reinterpret_cast<long long*>(sum_frame_dev);
  switch (elem_kind) {
    case 1:
      launch_count<uint8_t>(frames_dev, vec, thr_on, grid, st, nframes, npix, threshold, sb_counts_dev, sb_first_dev,
                            sb_before_dev, blk_totals_dev, sum);
      break;
    case -1:
      launch_count<int8_t>(frames_dev, vec, thr_on, grid, st, nframes, npix, threshold, sb_counts_dev, sb_first_dev,
                           sb_before_dev, blk_totals_dev, sum);
      break;
    case 2:
      launch_count<uint16_t>(frames_dev, vec, thr_on, grid, st, nframes, npix, threshold, sb_counts_dev,
                             sb_first_dev, sb_before_dev, blk_totals_dev, sum);
      break;
    default:
      launch_count<int16_t>(frames_dev, vec, thr_on, grid, st, nframes, npix, threshold, sb_counts_dev, sb_first_dev,
                            sb_before_dev, blk_totals_dev, sum);
  }
  return launch_status();
}

extern "C" int g2_compress_finish(uint16_t* sb_counts_dev, const uint16_t* sb_first_dev,
                                  const uint16_t* sb_before_dev, int32_t nframes, int64_t npix, uint8_t* mask_dev,
                                  uint32_t* blk_totals_dev, uint32_t* counts_dev, int32_t* t_cut_dev, void* stream) {
  if (!sb_counts_dev || !blk_totals_dev || !counts_dev || nframes <= 0 || npix <= 0) return G2_ERR_ARG;
  if ((sb_first_dev == nullptr) != (sb_before_dev == nullptr)) return G2_ERR_ARG;
  const int64_t n_sb = (static_cast<int64_t>(nframes) + cmp::SUBBLOCK - 1) / cmp::SUBBLOCK;
  const int64_t n_blk = (npix + cmp::BLK_PX - 1) / cmp::BLK_PX;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int blocks = n_blocks(npix, cmp::THREADS, sms, 16);
  cudaStream_t st = as_stream(stream);
  if (sb_first_dev)
    cmp::finish_kernel<true><<<blocks, cmp::THREADS, 0, st>>>(sb_counts_dev, sb_first_dev, sb_before_dev,
                                                              static_cast<int>(n_sb), nframes, npix, mask_dev,
                                                              blk_totals_dev, n_blk, counts_dev, t_cut_dev);
  else
    cmp::finish_kernel<false><<<blocks, cmp::THREADS, 0, st>>>(sb_counts_dev, nullptr, nullptr,
                                                               static_cast<int>(n_sb), nframes, npix, mask_dev,
                                                               blk_totals_dev, n_blk, counts_dev, t_cut_dev);
  return launch_status();
}

extern "C" int g2_compress_stage(const void* frames_dev, int32_t elem_kind, int32_t nframes, int64_t npix,
                                 const uint16_t* sb_counts_dev, const int32_t* t_cut_dev,
                                 const uint32_t* blk_base_dev, uint32_t* tile_pos_dev, uint32_t* stage_dev,
                                 int64_t n_stage, int32_t* err_dev, void* stream) {
  if (!frames_dev || !sb_counts_dev || !blk_base_dev || !tile_pos_dev || !stage_dev || !err_dev ||
      !kind_ok(elem_kind) || nframes <= 0 || npix <= 0 || n_stage < 0)
    return G2_ERR_ARG;
  if (n_stage >= (1ll << 32)) return G2_ERR_UNSUPPORTED;
  dim3 grid;
  const int rc = stack_grid(nframes, npix, grid);
  if (rc != G2_OK) return rc;
  const int64_t n_tiles = (npix + cmp::TILE_P - 1) / cmp::TILE_P;
  const int64_t eb = kind_bytes(elem_kind);
  const bool vec = npix % cmp::PX == 0 && aligned(frames_dev, static_cast<uintptr_t>(eb * cmp::PX));
  const bool cut_on = t_cut_dev != nullptr;
  cudaStream_t st = as_stream(stream);
  int lrc;
  switch (elem_kind) {
    case 1:
      lrc = launch_stage<uint8_t>(frames_dev, vec, cut_on, grid, st, nframes, npix, sb_counts_dev, t_cut_dev,
                             blk_base_dev, n_tiles, tile_pos_dev, stage_dev, n_stage, err_dev);
      break;
    case -1:
      lrc = launch_stage<int8_t>(frames_dev, vec, cut_on, grid, st, nframes, npix, sb_counts_dev, t_cut_dev,
                             blk_base_dev, n_tiles, tile_pos_dev, stage_dev, n_stage, err_dev);
      break;
    case 2:
      lrc = launch_stage<uint16_t>(frames_dev, vec, cut_on, grid, st, nframes, npix, sb_counts_dev, t_cut_dev,
                             blk_base_dev, n_tiles, tile_pos_dev, stage_dev, n_stage, err_dev);
      break;
    default:
      lrc = launch_stage<int16_t>(frames_dev, vec, cut_on, grid, st, nframes, npix, sb_counts_dev, t_cut_dev,
                             blk_base_dev, n_tiles, tile_pos_dev, stage_dev, n_stage, err_dev);
  }
  return lrc != G2_OK ? lrc : launch_status();
}

extern "C" int g2_stream_compress(const void* frames_dev, int32_t elem_kind, int32_t n_batch, int64_t frame0,
                                  int64_t npix, int32_t max_nnz, int32_t threshold, uint8_t* mask_dev,
                                  int64_t* sum_frame_dev, void* events_dev, int32_t* times_dev, int32_t* counter_dev,
                                  int32_t* err_dev, void* stream) {
  if (!frames_dev || !events_dev || !times_dev || !counter_dev || !err_dev || !kind_ok(elem_kind) || n_batch < 0 ||
      npix <= 0 || max_nnz <= 0 || frame0 < 0)
    return G2_ERR_ARG;
  if (n_batch == 0) return G2_OK;
  if (frame0 + n_batch > 0x7fffffffll) return G2_ERR_TOO_LARGE;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int blocks = n_blocks(npix, cmp::THREADS, sms, 16);
  cudaStream_t st = as_stream(stream);
  long long* sum = reinterpret_cast<long long*>(sum_frame_dev);
#define G2_SC(TV)                                                                                                \
  do {                                                                                                           \
    if (threshold >= 0)                                                                                          \
      cmp::stream_kernel<TV, true><<<blocks, cmp::THREADS, 0, st>>>(                                             \
          reinterpret_cast<const TV*>(frames_dev), n_batch, frame0, npix, max_nnz, threshold, mask_dev, sum,      \
          reinterpret_cast<TV*>(events_dev), times_dev, counter_dev, err_dev);                                   \
    else                                                                                                         \
      cmp::stream_kernel<TV, false><<<blocks, cmp::THREADS, 0, st>>>(                                            \
          reinterpret_cast<const TV*>(frames_dev), n_batch, frame0, npix, max_nnz, threshold, mask_dev, sum,      \
          reinterpret_cast<TV*>(events_dev), times_dev, counter_dev, err_dev);                                   \
  } while (0)
  switch (elem_kind) {
    case 1: G2_SC(uint8_t); break;
    case -1: G2_SC(int8_t); break;
    case 2: G2_SC(uint16_t); break;
    default: G2_SC(int16_t);
  }
#undef G2_SC
  return launch_status();
}

extern "C" int g2_stream_compact(const void* events_dev, const int32_t* times_dev, const int32_t* counter_dev,
                                 int32_t elem_bytes, int64_t npix, int32_t max_nnz, const uint32_t* offsets_dev,
                                 int64_t capacity, void* out_data_dev, int32_t* out_times_dev, int32_t* err_dev,
                                 void* stream) {
  if (!events_dev || !times_dev || !counter_dev || !offsets_dev || !out_data_dev || !out_times_dev || !err_dev ||
      (elem_bytes != 1 && elem_bytes != 2) || npix <= 0 || max_nnz <= 0 || capacity < 0)
    return G2_ERR_ARG;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int blocks = n_blocks(npix, cmp::THREADS, sms, 16);
  cudaStream_t st = as_stream(stream);
  if (elem_bytes == 1)
    cmp::compact_kernel<uint8_t><<<blocks, cmp::THREADS, 0, st>>>(
        reinterpret_cast<const uint8_t*>(events_dev), times_dev, counter_dev, npix, max_nnz, offsets_dev, capacity,
        reinterpret_cast<uint8_t*>(out_data_dev), out_times_dev, err_dev);
  else
    cmp::compact_kernel<uint16_t><<<blocks, cmp::THREADS, 0, st>>>(
        reinterpret_cast<const uint16_t*>(events_dev), times_dev, counter_dev, npix, max_nnz, offsets_dev, capacity,
        reinterpret_cast<uint16_t*>(out_data_dev), out_times_dev, err_dev);
  return launch_status();
}
