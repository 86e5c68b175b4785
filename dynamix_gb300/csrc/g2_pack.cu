// G1: gather each q-bin's pixels of every frame into the packed fp16 operand
// matrix of the Gram, and compute the per-frame bin sums S_b(t) on the way.
//
// The frames are read once; the packed matrix [T][packed_cols] is written
// once (bins are contiguous 64-column-padded segments).  Each thread owns
// four consecutive source columns of one 64-column segment (their pixel
// indices stay in registers for all frames) and handles FR frames per step.
// A half-warp covers one segment: its lanes reduce the segment's count sum
// (for S) and sum of squared packed values (for the exactness bound of the
// Gram's K split) with shuffles; one thread per block merges the segments of
// the same bin before the int64 atomic into S.
// Replaces compute_sums_dense (densecorrelator.cl:65-150) and the gather /
// float32 cast of py_dense_correlator (dense.py:48-50).
#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace pack {

constexpr int THREADS = 256;
constexpr int SEGS_PER_BLOCK = THREADS / 16;  // 16 threads x 4 columns = one 64-column segment
constexpr int FR = 4;                         // frames per step (loads in flight)

__device__ __forceinline__ uint32_t half_bits(uint32_t v) {
  return static_cast<uint32_t>(__half_as_ushort(__uint2half_rn(v)));
}
// e4m3 byte of an integer count 0..16 (exact in e4m3)
__device__ __forceinline__ uint32_t e4m3_bits(uint32_t v) {
  return static_cast<uint32_t>(__nv_cvt_float_to_fp8(static_cast<float>(v), __NV_SATFINITE, __NV_E4M3));
}

template <typename Tin>
__global__ void __launch_bounds__(THREADS)
    pack_kernel(const Tin* __restrict__ frames, int64_t T, int64_t npix, const int32_t* __restrict__ col_src,
                const int32_t* __restrict__ seg_bin, const int32_t* __restrict__ seg_dst0,
                const int32_t* __restrict__ seg_dst1, int64_t n_segs, int mode, uint8_t* __restrict__ packed,
                int64_t packed_cols, unsigned long long* __restrict__ sums, int n_bins,
                uint32_t* __restrict__ seg_emax, int32_t* __restrict__ err) {
  __shared__ unsigned long long s_sum[FR][SEGS_PER_BLOCK];
  __shared__ int s_bin[SEGS_PER_BLOCK];
  const int tid = threadIdx.x;
  const int lseg = tid >> 4;
  const int qd = tid & 15;
  const int64_t seg = static_cast<int64_t>(blockIdx.x) * SEGS_PER_BLOCK + lseg;
  const bool active = seg < n_segs;

  int32_t src[4] = {-1, -1, -1, -1};
  int bin = -1;
  int64_t dst0 = 0, dst1 = 0;
  if (active) {
    const int4 s4 = *reinterpret_cast<const int4*>(col_src + seg * 64 + qd * 4);
    src[0] = s4.x;
    src[1] = s4.y;
    src[2] = s4.z;
    src[3] = s4.w;
    bin = seg_bin[seg];
    dst0 = static_cast<int64_t>(seg_dst0[seg]) + qd * 4;
    dst1 = mode == 1 ? static_cast<int64_t>(seg_dst1[seg]) + qd * 4 : 0;
    bool bad = bin < 0 || bin >= n_bins || dst0 < 0 || dst0 + 4 > packed_cols ||
               (mode == 1 && (dst1 < 0 || dst1 + 4 > packed_cols));
    for (int k = 0; k < 4; ++k) bad |= src[k] >= npix;
    if (bad) {
      if (qd == 0) atomicOr(err, G2_DEVERR_BOUNDS);
      src[0] = src[1] = src[2] = src[3] = -1;
      bin = -1;
    }
  }
  const bool writes = active && bin >= 0;
  if (qd == 0) s_bin[lseg] = writes ? bin : -1;
  uint32_t emax0 = 0, emax1 = 0;
  uint32_t range_bad = 0;

  for (int64_t t0 = static_cast<int64_t>(blockIdx.y) * FR; t0 < T; t0 += static_cast<int64_t>(gridDim.y) * FR) {
    uint32_t v[FR][4];
#pragma unroll
    for (int f = 0; f < FR; ++f) {
      const int64_t t = t0 + f;
      const Tin* fr = frames + t * npix;
#pragma unroll
      for (int k = 0; k < 4; ++k) v[f][k] = (t < T && src[k] >= 0) ? static_cast<uint32_t>(fr[src[k]]) : 0u;
    }
#pragma unroll
    for (int f = 0; f < FR; ++f) {
      const int64_t t = t0 + f;
      uint32_t ssum = v[f][0] + v[f][1] + v[f][2] + v[f][3];
      uint32_t e0, e1 = 0;
      if (mode == 2) {
        e0 = v[f][0] * v[f][0] + v[f][1] * v[f][1] + v[f][2] * v[f][2] + v[f][3] * v[f][3];
        range_bad |= max(max(v[f][0], v[f][1]), max(v[f][2], v[f][3])) > 16u ? 1u : 0u;
        if (writes && t < T) {
          const uint32_t o = e4m3_bits(v[f][0]) | (e4m3_bits(v[f][1]) << 8) | (e4m3_bits(v[f][2]) << 16) |
                             (e4m3_bits(v[f][3]) << 24);
          *reinterpret_cast<uint32_t*>(packed + t * packed_cols + dst0) = o;
        }
      } else if (mode == 0) {
        e0 = v[f][0] * v[f][0] + v[f][1] * v[f][1] + v[f][2] * v[f][2] + v[f][3] * v[f][3];
        range_bad |= max(max(v[f][0], v[f][1]), max(v[f][2], v[f][3])) > 2048u ? 1u : 0u;
        if (writes && t < T) {
          uint2 o;
          o.x = half_bits(v[f][0]) | (half_bits(v[f][1]) << 16);
          o.y = half_bits(v[f][2]) | (half_bits(v[f][3]) << 16);
          *reinterpret_cast<uint2*>(packed + 2 * (t * packed_cols + dst0)) = o;
        }
      } else {
        uint32_t h[4], l[4];
        e0 = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          h[k] = v[f][k] >> 8;
          l[k] = v[f][k] & 255u;
          e0 += h[k] * h[k];
          e1 += l[k] * l[k];
          range_bad |= v[f][k] > 65535u ? 1u : 0u;
        }
        if (writes && t < T) {
          uint2 oh, ol;
          oh.x = half_bits(h[0]) | (half_bits(h[1]) << 16);
          oh.y = half_bits(h[2]) | (half_bits(h[3]) << 16);
          ol.x = half_bits(l[0]) | (half_bits(l[1]) << 16);
          ol.y = half_bits(l[2]) | (half_bits(l[3]) << 16);
          *reinterpret_cast<uint2*>(packed + 2 * (t * packed_cols + dst0)) = oh;
          *reinterpret_cast<uint2*>(packed + 2 * (t * packed_cols + dst1)) = ol;
        }
      }
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        ssum += __shfl_xor_sync(0xffffffffu, ssum, o);
        e0 += __shfl_xor_sync(0xffffffffu, e0, o);
        e1 += __shfl_xor_sync(0xffffffffu, e1, o);
      }
      if (qd == 0) {
        emax0 = max(emax0, e0);
        emax1 = max(emax1, e1);
        s_sum[f][lseg] = ssum;
      }
    }
    __syncthreads();
    if (tid < FR) {
      // merge consecutive segments of the same bin, one atomic per run
      const int f = tid;
      const int64_t t = t0 + f;
      if (t < T) {
        int cur = s_bin[0];
        unsigned long long acc = s_sum[f][0];
        for (int k = 1; k < SEGS_PER_BLOCK; ++k) {
          const int b = s_bin[k];
          if (b == cur) {
            acc += s_sum[f][k];
          } else {
            if (cur >= 0 && acc) atomicAdd(&sums[static_cast<int64_t>(cur) * T + t], acc);
            cur = b;
            acc = s_sum[f][k];
          }
        }
        if (cur >= 0 && acc) atomicAdd(&sums[static_cast<int64_t>(cur) * T + t], acc);
      }
    }
    __syncthreads();
  }
  if (writes && qd == 0) {
    if (emax0) atomicMax(&seg_emax[dst0 >> 6], emax0);
    if (mode == 1 && emax1) atomicMax(&seg_emax[dst1 >> 6], emax1);
  }
  if (range_bad) atomicOr(err, G2_DEVERR_RANGE);
}

template <typename Tin>
__global__ void binned_max_kernel(const Tin* __restrict__ frames, int64_t T, int64_t npix,
                                  const int32_t* __restrict__ col_src, int64_t n_cols, uint32_t* __restrict__ out) {
  uint32_t m = 0;
  const int64_t total = T * n_cols;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t t = i / n_cols;
    const int32_t s = col_src[i - t * n_cols];
    if (s >= 0 && s < npix) m = max(m, static_cast<uint32_t>(frames[t * npix + s]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

}  // namespace pack
}  // namespace g2

extern "C" int g2_pack_frames(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                              const int32_t* col_src_dev, const int32_t* seg_bin_dev, const int32_t* seg_dst0_dev,
                              const int32_t* seg_dst1_dev, int64_t n_segs, int32_t mode, void* packed_dev,
                              int64_t packed_cols, int64_t* sums_dev, int32_t n_bins, uint32_t* seg_emax_dev,
                              int32_t* err_dev, void* stream) {
  using namespace g2;
  if (!frames_dev || !col_src_dev || !seg_bin_dev || !seg_dst0_dev || !packed_dev || !sums_dev ||
      !seg_emax_dev || !err_dev)
    return G2_ERR_ARG;
  if ((elem_bytes != 1 && elem_bytes != 2) || nframes <= 0 || npix <= 0 || npix >= (1ll << 31) || n_segs < 0 ||
      mode < 0 || mode > 2 || (mode == 1 && !seg_dst1_dev) || packed_cols <= 0 || packed_cols % G2_PAD != 0 ||
      n_bins <= 0)
    return G2_ERR_ARG;
  if (!aligned(col_src_dev, 16) || !aligned(packed_dev, 16)) return G2_ERR_ARG;
  if (n_segs == 0) return G2_OK;
  const int64_t gx = (n_segs + pack::SEGS_PER_BLOCK - 1) / pack::SEGS_PER_BLOCK;
  if (gx > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  // enough blocks for ~8 resident per SM; each y-block walks frames with stride gy*FR
  int64_t gy = (static_cast<int64_t>(sms) * 8 + gx - 1) / gx;
  const int64_t max_gy = (nframes + pack::FR - 1) / pack::FR;
  if (gy > max_gy) gy = max_gy;
  if (gy > 65535) gy = 65535;
  if (gy < 1) gy = 1;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  auto* sums = reinterpret_cast<unsigned long long*>(sums_dev);
  auto* out = reinterpret_cast<uint8_t*>(packed_dev);
  if (elem_bytes == 1)
    pack::pack_kernel<uint8_t><<<grid, pack::THREADS, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint8_t*>(frames_dev), nframes, npix, col_src_dev, seg_bin_dev, seg_dst0_dev,
        seg_dst1_dev, n_segs, mode, out, packed_cols, sums, n_bins, seg_emax_dev, err_dev);
  else
    pack::pack_kernel<uint16_t><<<grid, pack::THREADS, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint16_t*>(frames_dev), nframes, npix, col_src_dev, seg_bin_dev, seg_dst0_dev,
        seg_dst1_dev, n_segs, mode, out, packed_cols, sums, n_bins, seg_emax_dev, err_dev);
  return launch_status();
}

extern "C" int g2_binned_max(const void* frames_dev, int32_t elem_bytes, int64_t nframes, int64_t npix,
                             const int32_t* col_src_dev, int64_t n_cols, uint32_t* max_dev, void* stream) {
  using namespace g2;
  if (!frames_dev || !col_src_dev || !max_dev || (elem_bytes != 1 && elem_bytes != 2) || nframes <= 0 ||
      npix <= 0 || n_cols < 0)
    return G2_ERR_ARG;
  if (n_cols == 0) return G2_OK;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const unsigned grid = static_cast<unsigned>(sms * 8);
  if (elem_bytes == 1)
    pack::binned_max_kernel<uint8_t><<<grid, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint8_t*>(frames_dev), nframes, npix, col_src_dev, n_cols, max_dev);
  else
    pack::binned_max_kernel<uint16_t><<<grid, 256, 0, as_stream(stream)>>>(
        reinterpret_cast<const uint16_t*>(frames_dev), nframes, npix, col_src_dev, n_cols, max_dev);
  return launch_status();
}
