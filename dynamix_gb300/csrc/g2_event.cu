// G6: event-list correlation -- integer pair sums over each pixel's events.
//
// Input layout of dynamix's EventCorrelator (event.py:267-284): for pixel p
// (flat index), events [offsets[p], offsets[p+1]) with frame times[e] and count
// data[e].  For every binned pixel and every pair of its events i <= j:
//     N_b(|t_j - t_i|) += v_i v_j,        S_b(t_i) += v_i.
// (evtcorrelator.cl:3-47 restated; the order of events within a pixel does not
// matter because the lag is |t_j - t_i|.)
//
// The host lists the binned pixels bin by bin (once per q-mask) and gives each
// CTA a contiguous slice of that list, cut into ranges of one bin each.  A CTA
// keeps the current bin's lag histogram and frame-sum histogram as uint32
// counters in shared memory (2 x T words) and flushes them at each range end.  A warp takes one pixel at a time, stages up to EV of its
// events in shared memory as (t << 16 | v) and walks the pairs: for each i (warp
// uniform) the lanes take j = i + lane, i + lane + 32, ...  A counter whose
// value reaches 2^31 is drained with an atomic exchange into the int64 global
// sums by the thread that saw it cross, so no uint32 counter can wrap (each
// increment is < 2^31 and at most a few thousand threads add concurrently).
// At the end the CTA adds its counters to the global N and S.
// When 2 T words do not fit in shared memory, or counts are large, a second
// kernel adds every pair directly to the global int64 sums.
#include <mutex>
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace ev {

constexpr int THREADS = 768;
constexpr int WARPS = THREADS / 32;
constexpr int LANES = 16;                  // lanes per pixel: a warp walks two pixels side by side
constexpr int HALVES = 32 / LANES;
constexpr int EV = 128;                    // events of one pixel staged per block of pairs
constexpr int ROWS = 8;                    // rows of the pair block walked together
constexpr uint32_t DRAIN = 1u << 31;
constexpr int SMEM_FIXED = WARPS * HALVES * 2 * EV * 4;
constexpr int SMEM_STATIC = WARPS * 8;    // block-reduction slots

__device__ __forceinline__ void add_counter(uint32_t* c, unsigned long long* g, uint32_t x) {
  const uint32_t old = atomicAdd(c, x);
  if (old + x >= DRAIN || old + x < old) {
    const uint32_t val = atomicExch(c, 0u);
    if (val) atomicAdd(g, static_cast<unsigned long long>(val));
  }
}

// One event as (t << 16) | v with its validity: from the caller's split
// arrays (times int32, data u8/u16) or from packed words (t << 16 | v).
template <bool PACKED, typename Tv>
__device__ __forceinline__ uint32_t load_event(const int32_t* __restrict__ times, const Tv* __restrict__ data,
                                               int64_t i, int T, uint32_t maxc, bool& ok) {
  if (PACKED) {
    const uint32_t w = reinterpret_cast<const uint32_t*>(times)[i];
    ok = static_cast<int>(w >> 16) < T && (w & 0xFFFFu) <= maxc;
    return w;
  }
  const int32_t t = times[i];
  const uint32_t v = static_cast<uint32_t>(data[i]);
  ok = t >= 0 && t < T && v <= maxc;
  return (static_cast<uint32_t>(t) << 16) | v;
}

// Pair sums of one pixel's events by one warp.  FAST: every counter of the
// range is known to stay below 2^32 (checked per range from its event count),
// so the shared adds need no returned value (the warp does not wait on them)
// and no drain check.
template <bool FAST, bool PACKED, typename Tv>
__device__ __forceinline__ void pixel_pairs(const int32_t* __restrict__ times, const Tv* __restrict__ data,
                                            int64_t base, int n, int T, uint32_t maxc, uint32_t* hist,
                                            uint32_t* shist, unsigned long long* gN, unsigned long long* gS,
                                            uint32_t* bufA, uint32_t* bufB, int lane, uint32_t mask, bool& bad) {
  for (int ib = 0; ib < n; ib += EV) {
    const int na = min(EV, n - ib);
    for (int e = lane; e < na; e += LANES) {
      bool ok;
      const uint32_t w = load_event<PACKED>(times, data, base + ib + e, T, maxc, ok);
      const int t = static_cast<int>(w >> 16);
      const uint32_t v = w & 0xFFFFu;
      bad |= !ok;
      bufA[e] = ok ? w : 0u;
      if (ok && v) {
        if (FAST)
          atomicAdd(&shist[t], v);
        else
          add_counter(&shist[t], &gS[t], v);
      }
    }
    __syncwarp(mask);
    for (int jb = ib; jb < n; jb += EV) {
      const int nb = min(EV, n - jb);
      const uint32_t* B = bufA;
      if (jb != ib) {
        for (int e = lane; e < nb; e += LANES) {
          bool ok;
          const uint32_t w = load_event<PACKED>(times, data, base + jb + e, T, maxc, ok);
          bufB[e] = ok ? w : 0u;
        }
        __syncwarp(mask);
        B = bufB;
      }
      // ROWS rows (i .. i + ROWS - 1) per pass: each partner word read from
      // shared memory serves ROWS pairs, and the row overhead is paid once
      // per ROWS rows.  Absent rows and pairs below the diagonal get a zero
      // product, whose unconditional add changes nothing.
      const bool tri = jb == ib;
      for (int i = 0; i < na; i += ROWS) {
        uint32_t vi[ROWS];
        int ti[ROWS];
        uint32_t any = 0;
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
          const uint32_t w = i + r < na ? bufA[i + r] : 0u;
          vi[r] = w & 0xFFFFu;
          ti[r] = static_cast<int>(w >> 16);
          any |= vi[r];
        }
        if (any == 0) continue;  // warp-uniform
        for (int j = (tri ? i : 0) + lane; j < nb; j += LANES) {
          const uint32_t wj = B[j];
          const int tj = static_cast<int>(wj >> 16);
          const uint32_t vj = wj & 0xFFFFu;
#pragma unroll
          for (int r = 0; r < ROWS; ++r) {
            const uint32_t prod = (!tri || j >= i + r) ? vi[r] * vj : 0u;  // the diagonal block takes j >= i + r
            const int lag = abs(tj - ti[r]);
            if (FAST)
              atomicAdd(&hist[lag], prod);
            else if (prod)
              add_counter(&hist[lag], &gN[lag], prod);
          }
        }
      }
      __syncwarp(mask);
    }
  }
}

template <bool PACKED, typename Tv>
__global__ void __launch_bounds__(THREADS, 1)
    pairs_smem_kernel(const int32_t* __restrict__ times, const Tv* __restrict__ data,
                      const uint32_t* __restrict__ offsets, const int32_t* __restrict__ pix_list,
                      const int32_t* __restrict__ range_off, const int32_t* __restrict__ range_bin,
                      const int32_t* __restrict__ cta_range_off, int n_ranges, int64_t n_events,
                      int64_t npix, int32_t T, int n_bins, uint32_t maxc, unsigned long long* __restrict__ numer,
                      unsigned long long* __restrict__ sums, int32_t* __restrict__ err) {
  extern __shared__ __align__(16) uint32_t sm[];
  __shared__ unsigned long long s_red[WARPS];
  uint32_t* hist = sm;              // [T] lag sums of this range's bin
  uint32_t* shist = sm + T;         // [T] frame sums
  uint32_t* evbuf = sm + 2 * T;     // [WARPS][HALVES][2][EV] staged events (t << 16 | v)
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane / LANES, hl = lane % LANES;
  const uint32_t hmask = (LANES == 32 ? 0xffffffffu : ((1u << LANES) - 1u)) << (half * LANES);
  uint32_t* bufA = evbuf + (warp * HALVES + half) * 2 * EV;
  uint32_t* bufB = bufA + EV;
  bool bad = false;
  for (int i = threadIdx.x; i < 2 * T; i += THREADS) sm[i] = 0;
  const unsigned long long max2 = static_cast<unsigned long long>(maxc) * maxc;
  // this CTA's ranges (a contiguous slice of the bin-ordered pixel list, cut
  // at bin boundaries); the counters are flushed once per range
  const int r_end = min(cta_range_off[blockIdx.x + 1], n_ranges);
  for (int r = max(cta_range_off[blockIdx.x], 0); r < r_end; ++r) {
    const int bin = range_bin[r];
    if (bin < 0 || bin >= n_bins) {
      bad = true;
      continue;  // uniform over the CTA
    }
    // events of the range: a lag counter gains at most max^2 per event and a
    // frame counter at most max per pixel, so max^2 * events < 2^32 keeps
    // every counter of the range in uint32 without draining
    unsigned long long ev = 0;
    for (int li = range_off[r] + threadIdx.x; li < range_off[r + 1]; li += THREADS) {
      const int32_t p = pix_list[li];
      if (p >= 0 && p < npix) {
        const uint32_t a = offsets[p], b = offsets[p + 1];
        if (b >= a) ev += b - a;
      }
    }
    for (int o = 16; o; o >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, o);
    if (lane == 0) s_red[warp] = ev;
    __syncthreads();  // also: counters zeroed (start, or the previous flush)
    unsigned long long tot = 0;
    for (int w = 0; w < WARPS; ++w) tot += s_red[w];
    const bool fast = max2 == 0 || tot < (1ull << 32) / max2;
    unsigned long long* gN = numer + static_cast<int64_t>(bin) * T;
    unsigned long long* gS = sums + static_cast<int64_t>(bin) * T;
    // each half-warp takes its own pixel (its own staging buffers; it syncs
    // only its own lanes), so that a pixel's pair rows leave half as many
    // lanes idle at their ends as 32-lane rows would
    for (int li = range_off[r] + warp * HALVES + half; li < range_off[r + 1]; li += WARPS * HALVES) {
      const int32_t p = pix_list[li];
      if (p < 0 || p >= npix) {
        bad = true;
        continue;
      }
      const int64_t base = offsets[p];
      const int64_t end = offsets[p + 1];
      if (end < base || end > n_events) {
        bad = true;
        continue;
      }
      const int n = static_cast<int>(end - base);
      if (fast)
        pixel_pairs<true, PACKED>(times, data, base, n, T, maxc, hist, shist, gN, gS, bufA, bufB, hl, hmask, bad);
      else
        pixel_pairs<false, PACKED>(times, data, base, n, T, maxc, hist, shist, gN, gS, bufA, bufB, hl, hmask, bad);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < T; i += THREADS) {
      const uint32_t h = hist[i], sh = shist[i];
      if (h) atomicAdd(&gN[i], static_cast<unsigned long long>(h));
      if (sh) atomicAdd(&gS[i], static_cast<unsigned long long>(sh));
      hist[i] = 0;
      shist[i] = 0;
    }
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

// Every pair added straight to the global int64 sums (long stacks, large counts).
template <bool PACKED, typename Tv>
__global__ void __launch_bounds__(256)
    pairs_global_kernel(const int32_t* __restrict__ times, const Tv* __restrict__ data,
                        const uint32_t* __restrict__ offsets, const int32_t* __restrict__ pix_list,
                        const int32_t* __restrict__ range_off, const int32_t* __restrict__ range_bin,
                        const int32_t* __restrict__ cta_range_off, int n_ranges, int64_t n_events, int64_t npix,
                        int32_t T,
                        int n_bins,
                        unsigned long long* __restrict__ numer, unsigned long long* __restrict__ sums,
                        int32_t* __restrict__ err) {
  const int warps = blockDim.x >> 5;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  bool bad = false;
  const int r_end = min(cta_range_off[blockIdx.x + 1], n_ranges);
  for (int r = max(cta_range_off[blockIdx.x], 0); r < r_end; ++r) {
  const int bin = range_bin[r];
  if (bin < 0 || bin >= n_bins) {
    bad = true;
    continue;
  }
  unsigned long long* gN = numer + static_cast<int64_t>(bin) * T;
  unsigned long long* gS = sums + static_cast<int64_t>(bin) * T;
  for (int li = range_off[r] + warp; li < range_off[r + 1]; li += warps) {
    const int32_t p = pix_list[li];
    if (p < 0 || p >= npix) {
      bad = true;
      continue;
    }
    const int64_t base = offsets[p];
    const int64_t end = offsets[p + 1];
    if (end < base || end > n_events) {
      bad = true;
      continue;
    }
    const int64_t n = end - base;
    for (int64_t i = 0; i < n; ++i) {
      bool oki;
      const uint32_t wi = load_event<PACKED>(times, data, base + i, T, 0xFFFFu, oki);
      const int32_t ti = static_cast<int32_t>(wi >> 16);
      const unsigned long long vi = wi & 0xFFFFu;
      if (!oki) {
        bad = true;
        continue;
      }
      if (lane == 0 && vi) atomicAdd(&gS[ti], vi);
      if (!vi) continue;
      for (int64_t j = i + lane; j < n; j += 32) {
        bool okj;
        const uint32_t wj = load_event<PACKED>(times, data, base + j, T, 0xFFFFu, okj);
        const int32_t tj = static_cast<int32_t>(wj >> 16);
        const unsigned long long vj = wj & 0xFFFFu;
        if (!okj || !vj) continue;
        atomicAdd(&gN[abs(tj - ti)], vi * vj);
      }
    }
  }
  }
  if (bad) atomicOr(err, G2_DEVERR_BOUNDS);
}

}  // namespace ev
}  // namespace g2

namespace {
template <bool PACKED>
int pairsum(const int32_t* times_dev, const void* data_dev, int32_t elem_bytes, int64_t n_events,
            const uint32_t* offsets_dev, int64_t npix, const int32_t* pix_list_dev, const int32_t* range_off_dev,
            const int32_t* range_bin_dev, int32_t n_ranges, const int32_t* cta_range_off_dev, int32_t n_ctas,
            int32_t nframes, int32_t n_bins, int32_t max_count, uint64_t* numer_dev, uint64_t* sums_dev,
            int32_t* err_dev, void* stream) {
  using namespace g2;
  if (n_ranges == 0 || n_ctas <= 0) return G2_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return G2_ERR_CUDA;
  int smem_optin = 0;
  if (cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return G2_ERR_CUDA;
  const int64_t smem = static_cast<int64_t>(nframes) * 8 + ev::SMEM_FIXED;
  // shared counters need t < 2^16 (packed with the count) and products < 2^31
  const bool use_smem = smem + ev::SMEM_STATIC <= smem_optin && nframes <= 65535 &&
                        static_cast<int64_t>(max_count) * max_count < (1ll << 31);
  auto* N = reinterpret_cast<unsigned long long*>(numer_dev);
  auto* S = reinterpret_cast<unsigned long long*>(sums_dev);
  cudaStream_t st = as_stream(stream);
  const uint32_t maxc = static_cast<uint32_t>(max_count);
#define G2_PAIRS(TV)                                                                                              \
  do {                                                                                                            \
    const TV* d = reinterpret_cast<const TV*>(data_dev);                                                          \
    if (use_smem) {                                                                                               \
      if (cudaFuncSetAttribute(ev::pairs_smem_kernel<PACKED, TV>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                               static_cast<int>(smem)) != cudaSuccess)                                            \
        return G2_ERR_CUDA;                                                                                       \
      ev::pairs_smem_kernel<PACKED, TV><<<n_ctas, ev::THREADS, smem, st>>>(                                       \
          times_dev, d, offsets_dev, pix_list_dev, range_off_dev, range_bin_dev, cta_range_off_dev, n_ranges,     \
          n_events, npix, nframes, n_bins, maxc, N, S, err_dev);                                                  \
    } else {                                                                                                      \
      ev::pairs_global_kernel<PACKED, TV><<<n_ctas, 256, 0, st>>>(times_dev, d, offsets_dev, pix_list_dev,       \
                                                                  range_off_dev, range_bin_dev, cta_range_off_dev, \
                                                                  n_ranges, n_events, npix, nframes, n_bins, N, S, \
                                                                  err_dev);                                       \
    }                                                                                                             \
  } while (0)
  if (elem_bytes == 1)
    G2_PAIRS(uint8_t);
  else
    G2_PAIRS(uint16_t);
#undef G2_PAIRS
  return launch_status();
}
}  // namespace

extern "C" int g2_event_pairsum(const int32_t* times_dev, const void* data_dev, int32_t elem_bytes,
                                int64_t n_events, const uint32_t* offsets_dev, int64_t npix,
                                const int32_t* pix_list_dev, const int32_t* range_off_dev,
                                const int32_t* range_bin_dev, int32_t n_ranges, const int32_t* cta_range_off_dev,
                                int32_t n_ctas, int32_t nframes, int32_t n_bins,
                                int32_t max_count, uint64_t* numer_dev, uint64_t* sums_dev, int32_t* err_dev,
                                void* stream) {
  using namespace g2;
  if (!times_dev || !data_dev || !offsets_dev || !pix_list_dev || !range_off_dev || !range_bin_dev ||
      !cta_range_off_dev || !numer_dev || !sums_dev || !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || n_events < 0 || npix <= 0 || n_ranges < 0 || nframes <= 0 ||
      n_bins <= 0 || max_count < 0 || max_count > 65535)
    return G2_ERR_ARG;
  return pairsum<false>(times_dev, data_dev, elem_bytes, n_events, offsets_dev, npix, pix_list_dev, range_off_dev,
                        range_bin_dev, n_ranges, cta_range_off_dev, n_ctas, nframes, n_bins, max_count, numer_dev,
                        sums_dev, err_dev, stream);
}

extern "C" int g2_event_pairsum_packed(const uint32_t* words_dev, int64_t n_events, const uint32_t* offsets_dev,
                                       int64_t npix, const int32_t* pix_list_dev, const int32_t* range_off_dev,
                                       const int32_t* range_bin_dev, int32_t n_ranges,
                                       const int32_t* cta_range_off_dev, int32_t n_ctas, int32_t nframes,
                                       int32_t n_bins, int32_t max_count, uint64_t* numer_dev, uint64_t* sums_dev,
                                       int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!words_dev || !offsets_dev || !pix_list_dev || !range_off_dev || !range_bin_dev || !cta_range_off_dev ||
      !numer_dev || !sums_dev || !err_dev)
    return G2_ERR_ARG;
  if (n_events < 0 || npix <= 0 || n_ranges < 0 || nframes <= 0 || nframes > 65536 || n_bins <= 0 ||
      max_count < 0 || max_count > 65535)
    return G2_ERR_ARG;
  // the data pointer is unused on the packed path; elem_bytes 1 selects one instantiation
  return pairsum<true>(reinterpret_cast<const int32_t*>(words_dev), words_dev, 1, n_events, offsets_dev, npix,
                       pix_list_dev, range_off_dev, range_bin_dev, n_ranges, cta_range_off_dev, n_ctas, nframes,
                       n_bins, max_count, numer_dev, sums_dev, err_dev, stream);
}
