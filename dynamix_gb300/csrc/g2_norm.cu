// G3 (denominator) and G4 (finalize).
//
// G3: D[r][tau] = sum_t S[r][t] * S[r][t+tau] in int64 for every row r (one row
// per (job, bin)).  A block owns 1024 lags of one row (4 consecutive per
// thread) and walks t in shared-memory windows of 1024 frames; the shifted
// window is padded with zeros beyond T, so no per-term bounds test is needed,
// and stored with one pad word per 32 so the threads' 4-word stride stays
// free of bank conflicts.
// Replaces correlate_1D (densecorrelator.cl:156-176), the sum loop of
// normalize_correlation (evtcorrelator.cl:70-73) and the mean outer product
// of py_dense_correlator (dense.py:55, :63).
//
// G4: g2 = scale * N / D in float64 (the only float64 arithmetic on the GPU),
// written as float32 and/or float64.  0/0 gives NaN as in the reference.
// Replaces densecorrelator.cl:54, evtcorrelator.cl:75 and dense.py:64.
#include <mutex>
#include "g2_ptx.cuh"
#include "g2_host.h"

namespace g2 {
namespace norm {

constexpr int THR = 256;
constexpr int LPT = 4;               // lags per thread, strided by THR
constexpr int LAGS = THR * LPT;      // lags per block
constexpr int WIN = 1024;            // frames per shared window

// S values are split into 32-bit halves in shared memory.  A window whose
// largest value m is below 2^16 accumulates in 32 bits, added to the 64-bit
// sums every (2^32 - 1) / m^2 frames.  Otherwise, windows whose
// values all fit in 32 bits (the usual case: a bin sum is at most
// pixels x max count) take one 32 x 32 -> 64-bit multiply-add per term;
// others add the cross terms too (arithmetic mod 2^64, exact while D < 2^63,
// which the host checks).
// Padded index of the shifted window: one pad word per 32, so lanes 4 words
// apart (a thread's 4 consecutive lags) fall on distinct banks.
__device__ __forceinline__ int pad32(int x) { return x + (x >> 5); }
constexpr int WIN2_PAD = WIN + LAGS + (WIN + LAGS) / 32;

__global__ void __launch_bounds__(THR)
    denom_kernel(const long long* __restrict__ S, int64_t T, long long* __restrict__ D) {
  __shared__ uint32_t lo1[WIN], hi1[WIN];
  __shared__ uint32_t lo2[WIN2_PAD], hi2[WIN2_PAD];
  __shared__ uint32_t s_wmax[THR / 32];
  const int64_t r = blockIdx.y;
  const int64_t tau0 = static_cast<int64_t>(blockIdx.x) * LAGS;
  const long long* row = S + r * T;
  const int l0 = LPT * threadIdx.x;  // this thread's lags: tau0 + l0 + k
  unsigned long long acc[LPT] = {0, 0, 0, 0};
  // split z of gridDim.z takes every gridDim.z-th window of frames
  for (int64_t t0 = static_cast<int64_t>(blockIdx.z) * WIN; t0 < T - tau0;
       t0 += static_cast<int64_t>(gridDim.z) * WIN) {
    bool wide = false;
    uint32_t vmax = 0;
    for (int i = threadIdx.x; i < WIN; i += THR) {
      const int64_t t = t0 + i;
      const unsigned long long v = t < T ? static_cast<unsigned long long>(row[t]) : 0ull;
      lo1[i] = static_cast<uint32_t>(v);
      hi1[i] = static_cast<uint32_t>(v >> 32);
      wide |= (v >> 32) != 0;
      vmax = max(vmax, static_cast<uint32_t>(v));
    }
    for (int i = threadIdx.x; i < WIN + LAGS; i += THR) {
      const int64_t t = t0 + tau0 + i;
      const unsigned long long v = t < T ? static_cast<unsigned long long>(row[t]) : 0ull;
      lo2[pad32(i)] = static_cast<uint32_t>(v);
      hi2[pad32(i)] = static_cast<uint32_t>(v >> 32);
      wide |= (v >> 32) != 0;
      vmax = max(vmax, static_cast<uint32_t>(v));
    }
    vmax = __reduce_max_sync(0xffffffffu, vmax);
    if ((threadIdx.x & 31) == 0) s_wmax[threadIdx.x >> 5] = vmax;  // read after the barrier below
    const int n = static_cast<int>(T - tau0 - t0 < WIN ? T - tau0 - t0 : WIN);  // terms with t + tau0 < T
    const bool any_wide = __syncthreads_or(wide);
    uint32_t wmax = 0;
#pragma unroll
    for (int w = 0; w < THR / 32; ++w) wmax = max(wmax, s_wmax[w]);
    // frames whose products sum below 2^32: (2^32 - 1) / max^2 (0 when one
    // product may not fit 32 bits)
    const unsigned long long m2 = static_cast<unsigned long long>(wmax) * wmax;
    const int run32 = m2 == 0 ? n : static_cast<int>(min(0xFFFFFFFFull / m2, static_cast<unsigned long long>(n)));
    if (!any_wide && run32 > 0) {
      // 32-bit multiply-adds, added to the 64-bit sums every run32 frames; the
      // shifted values b[k] = S(t + tau0 + l0 + k) slide along in registers,
      // one shared load per four multiply-adds
      uint32_t bv[LPT];
#pragma unroll
      for (int k = 0; k < LPT - 1; ++k) bv[k + 1] = lo2[pad32(l0 + k)];
      for (int i0 = 0; i0 < n; i0 += run32) {
        const int i1 = min(n, i0 + run32);
        uint32_t part[LPT] = {0, 0, 0, 0};
#pragma unroll 4
        for (int i = i0; i < i1; ++i) {
          const uint32_t a = lo1[i];
#pragma unroll
          for (int k = 0; k < LPT - 1; ++k) bv[k] = bv[k + 1];
          bv[LPT - 1] = lo2[pad32(i + l0 + LPT - 1)];
#pragma unroll
          for (int k = 0; k < LPT; ++k) part[k] += a * bv[k];
        }
#pragma unroll
        for (int k = 0; k < LPT; ++k) acc[k] += part[k];
      }
    } else if (any_wide) {
      for (int i = 0; i < n; ++i) {
        const unsigned long long a_lo = lo1[i], a_hi = hi1[i];
#pragma unroll
        for (int k = 0; k < LPT; ++k) {
          const int j = pad32(i + l0 + k);
          acc[k] += a_lo * lo2[j] + ((a_hi * lo2[j] + a_lo * hi2[j]) << 32);
        }
      }
    } else {
#pragma unroll 4
      for (int i = 0; i < n; ++i) {
        const uint32_t a = lo1[i];
#pragma unroll
        for (int k = 0; k < LPT; ++k) acc[k] += static_cast<unsigned long long>(a) * lo2[pad32(i + l0 + k)];
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int k = 0; k < LPT; ++k) {
    const int64_t tau = tau0 + l0 + k;
    if (tau < T) {
      if (gridDim.z == 1)
        D[r * T + tau] = static_cast<long long>(acc[k]);
      else if (acc[k])
        atomicAdd(reinterpret_cast<unsigned long long*>(&D[r * T + tau]), acc[k]);  // D zeroed by the host
    }
  }
}

// Launch G3 with enough blocks to fill the GPU: the frame windows are split
// over gridDim.z and the partial sums added atomically (mod 2^64, exact).
// The work of a lag block falls with its lags (fewer frames pair up), so the
// first blocks set the time: z aims at 32 blocks per SM, not just enough to
// occupy every SM (2162x2068x20k events, 32 bins: 1.01 -> 0.71 ms).
inline int launch_denominator(const long long* S, int32_t n_rows, int64_t T, long long* D, cudaStream_t st) {
  const int64_t gx = (T + LAGS - 1) / LAGS;
  if (gx > 0x7fffffff) return G2_ERR_TOO_LARGE;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int64_t windows = (T + WIN - 1) / WIN;
  int64_t z = (32ll * sms + gx * n_rows - 1) / (gx * n_rows);
  z = z < 1 ? 1 : (z > windows ? windows : (z > 32 ? 32 : z));
  if (z > 1 && cudaMemsetAsync(D, 0, static_cast<size_t>(n_rows) * T * sizeof(long long), st) != cudaSuccess)
    return G2_ERR_CUDA;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(n_rows), static_cast<unsigned>(z));
  denom_kernel<<<grid, THR, 0, st>>>(S, T, D);
  return launch_status();
}

__global__ void finalize_kernel(const long long* __restrict__ N, const long long* __restrict__ D,
                                const double* __restrict__ scale, int64_t rows, int64_t T, float* __restrict__ g32,
                                double* __restrict__ g64) {
  const int64_t total = rows * T;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t r = i / T;
    const double g = scale[r] * static_cast<double>(N[i]) / static_cast<double>(D[i]);
    if (g32) g32[i] = static_cast<float>(g);
    if (g64) g64[i] = g;
  }
}

// calc_std deviation (dense.py:58-66): dev(tau) = std_t(r) / sqrt(T - tau),
// from the sums of d = r - centre and d^2 over the T - tau pairs of the lag
// (population variance, as numpy's std); NaN when a pair had S(t) S(t') = 0
// (the reference divides by zero there).
__global__ void std_finalize_kernel(const double* __restrict__ sum_d, const double* __restrict__ sum_d2,
                                    const unsigned int* __restrict__ zeros, int64_t rows, int64_t T,
                                    float* __restrict__ d32, double* __restrict__ d64) {
  const int64_t total = rows * T;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double n = static_cast<double>(T - i % T);
    const double m = sum_d[i] / n;
    const double var = fmax(sum_d2[i] / n - m * m, 0.0);
    const double dev = zeros[i] ? __longlong_as_double(0x7ff8000000000000ll) : sqrt(var) / sqrt(n);
    if (d32) d32[i] = static_cast<float>(dev);
    if (d64) d64[i] = dev;
  }
}

// Deviation statistics of one bin from its Gram matrix G[t][t'] (t' >= t,
// row stride ld): for every pair, r = P G / (S(t) S(t')) and d = r - centre(tau)
// (0 when the centre is not finite), summed per lag in double into sum_d and
// sum_d2; pairs with S(t) S(t') = 0 are counted in zeros.  A block owns 256
// consecutive lags (a thread each, so that the loads of a row are
// coalesced) and a range of rows; one double atomic per lag per block.
__global__ void __launch_bounds__(256)
    matrix_deviation_kernel(const float* __restrict__ G, int64_t T, int64_t ld, const long long* __restrict__ S,
                            double P, const float* __restrict__ centre, double* __restrict__ sum_d,
                            double* __restrict__ sum_d2, unsigned int* __restrict__ zeros, int64_t rows_per_block) {
  const int64_t tau = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (tau >= T) return;
  const float cf = centre[tau];
  const double c = isfinite(cf) ? static_cast<double>(cf) : 0.0;
  const int64_t t0 = static_cast<int64_t>(blockIdx.y) * rows_per_block;
  int64_t t1 = t0 + rows_per_block;
  if (t1 > T - tau) t1 = T - tau;
  double sd = 0.0, sd2 = 0.0;
  unsigned int nz = 0;
  for (int64_t t = t0; t < t1; ++t) {
    const double den = static_cast<double>(S[t]) * static_cast<double>(S[t + tau]);
    if (den == 0.0) {
      ++nz;
    } else {
      const double d = P * static_cast<double>(G[t * ld + t + tau]) / den - c;
      sd += d;
      sd2 += d * d;
    }
  }
  if (t1 > t0) {
    if (sd != 0.0) atomicAdd(&sum_d[tau], sd);
    if (sd2 != 0.0) atomicAdd(&sum_d2[tau], sd2);
    if (nz) atomicAdd(&zeros[tau], nz);
  }
}

}  // namespace norm
}  // namespace g2

extern "C" int g2_matrix_deviation(const float* matrix_dev, int64_t nframes, int64_t ld, const int64_t* bin_sums_dev,
                                   double npix, const float* centre_dev, double* sum_d_dev, double* sum_d2_dev,
                                   uint32_t* zeros_dev, void* stream) {
  using namespace g2;
  if (!matrix_dev || !bin_sums_dev || !centre_dev || !sum_d_dev || !sum_d2_dev || !zeros_dev || nframes <= 0 ||
      ld < nframes || !(npix > 0.0))
    return G2_ERR_ARG;
  const int64_t rows_per_block = 256;
  const int64_t gx = (nframes + 255) / 256, gy = (nframes + rows_per_block - 1) / rows_per_block;
  if (gx > 0x7fffffff || gy > 65535) return G2_ERR_TOO_LARGE;
  norm::matrix_deviation_kernel<<<dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy)), 256, 0,
                                  as_stream(stream)>>>(matrix_dev, nframes, ld,
                                                       reinterpret_cast<const long long*>(bin_sums_dev), npix,
                                                       centre_dev, sum_d_dev, sum_d2_dev, zeros_dev, rows_per_block);
  return launch_status();
}

extern "C" int g2_std_finalize(const double* sum_d_dev, const double* sum_d2_dev, const uint32_t* zeros_dev,
                               int32_t n_rows, int64_t nframes, float* dev_f32, double* dev_f64, void* stream) {
  using namespace g2;
  if (!sum_d_dev || !sum_d2_dev || !zeros_dev || n_rows < 0 || nframes <= 0 || (!dev_f32 && !dev_f64))
    return G2_ERR_ARG;
  if (n_rows == 0) return G2_OK;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int64_t total = static_cast<int64_t>(n_rows) * nframes;
  int64_t blocks = (total + 255) / 256;
  if (blocks > sms * 8) blocks = sms * 8;
  norm::std_finalize_kernel<<<static_cast<unsigned>(blocks), 256, 0, as_stream(stream)>>>(
      sum_d_dev, sum_d2_dev, zeros_dev, n_rows, nframes, dev_f32, dev_f64);
  return launch_status();
}

extern "C" int g2_denominator(const int64_t* sums_dev, int32_t n_rows, int64_t nframes, int64_t* denom_dev,
                              void* stream) {
  using namespace g2;
  if (!sums_dev || !denom_dev || n_rows < 0 || nframes <= 0) return G2_ERR_ARG;
  if (n_rows == 0) return G2_OK;
  if (n_rows > 65535) return G2_ERR_TOO_LARGE;
  return norm::launch_denominator(reinterpret_cast<const long long*>(sums_dev), n_rows, nframes,
                                  reinterpret_cast<long long*>(denom_dev), as_stream(stream));
}

extern "C" int g2_finalize(const int64_t* numer_dev, const int64_t* denom_dev, const double* scale_dev,
                           int32_t n_rows, int64_t nframes, float* g2_f32_dev, double* g2_f64_dev, void* stream) {
  using namespace g2;
  if (!numer_dev || !denom_dev || !scale_dev || n_rows < 0 || nframes <= 0 || (!g2_f32_dev && !g2_f64_dev))
    return G2_ERR_ARG;
  if (n_rows == 0) return G2_OK;
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int64_t total = static_cast<int64_t>(n_rows) * nframes;
  int64_t blocks = (total + 255) / 256;
  if (blocks > sms * 8) blocks = sms * 8;
  norm::finalize_kernel<<<static_cast<unsigned>(blocks), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const long long*>(numer_dev), reinterpret_cast<const long long*>(denom_dev), scale_dev,
      n_rows, nframes, g2_f32_dev, g2_f64_dev);
  return launch_status();
}

// ---- G3+G4 for callers that cannot allocate ---------------------------------
// The denominator is kept in this file-scope device array instead of a
// caller-allocated buffer.  Host code must not pass the symbol itself to a
// kernel (on the host it names a stand-in, not device memory): the device
// address is looked up once per device with cudaGetSymbolAddress.
static __device__ __align__(256) long long g2_static_denom[G2_STATIC_DENOM_MAX];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
long long* g_static_denom_addr[kMaxDevices] = {};
}  // namespace

extern "C" int g2_normalize_static(const int64_t* numer_dev, const int64_t* sums_dev, const double* scale_dev,
                                   int32_t n_rows, int64_t nframes, float* g2_f32_dev, double* g2_f64_dev,
                                   void* stream) {
  using namespace g2;
  if (!numer_dev || !sums_dev || !scale_dev || n_rows < 0 || nframes <= 0 || (!g2_f32_dev && !g2_f64_dev))
    return G2_ERR_ARG;
  if (n_rows == 0) return G2_OK;
  if (static_cast<int64_t>(n_rows) * nframes > G2_STATIC_DENOM_MAX) return G2_ERR_TOO_LARGE;
  if (n_rows > 65535) return G2_ERR_TOO_LARGE;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return G2_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return G2_ERR_UNSUPPORTED;
  long long* denom = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_denom_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g2_static_denom) != cudaSuccess || p == nullptr) return G2_ERR_CUDA;
      g_static_denom_addr[dev] = static_cast<long long*>(p);
    }
    denom = g_static_denom_addr[dev];
  }
  const int sms = sm_count_current();
  if (sms <= 0) return G2_ERR_CUDA;
  const int64_t gx = (nframes + norm::LAGS - 1) / norm::LAGS;
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(n_rows));
  norm::denom_kernel<<<grid, norm::THR, 0, as_stream(stream)>>>(reinterpret_cast<const long long*>(sums_dev),
                                                                 nframes, denom);
  const int64_t total = static_cast<int64_t>(n_rows) * nframes;
  int64_t blocks = (total + 255) / 256;
  if (blocks > sms * 8) blocks = sms * 8;
  norm::finalize_kernel<<<static_cast<unsigned>(blocks), 256, 0, as_stream(stream)>>>(
      reinterpret_cast<const long long*>(numer_dev), denom, scale_dev, n_rows, nframes, g2_f32_dev, g2_f64_dev);
  return launch_status();
}
