// Host utilities of the C ABI: status strings, device queries, tensor maps.
#include <algorithm>
#include <cstring>
#include <functional>
#include <mutex>
#include <numeric>
#include <queue>
#include <utility>
#include <vector>
#include <cudaTypedefs.h>
#include "g2_host.h"

namespace g2 {

namespace {
std::mutex g_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
int g_sm_count[64] = {0};
}  // namespace

int sm_count_current() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (dev >= 0 && dev < 64 && g_sm_count[dev] > 0) return g_sm_count[dev];
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (dev >= 0 && dev < 64) g_sm_count[dev] = n;
  return n;
}

int encode_tmap_2d(CUtensorMap* map, const void* base, int elem_bytes, uint64_t cols, uint64_t rows,
                   uint32_t box_cols, uint32_t box_rows) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_encode) {
      void* fn = nullptr;
      cudaDriverEntryPointQueryResult q;
      if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
              cudaSuccess ||
          q != cudaDriverEntryPointSuccess || fn == nullptr)
        return G2_ERR_UNSUPPORTED;
      g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
  }
  const cuuint64_t dims[2] = {cols, rows};
  const cuuint64_t strides[1] = {cols * static_cast<uint64_t>(elem_bytes)};
  const cuuint32_t box[2] = {box_cols, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUtensorMapDataType dt = elem_bytes == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
  CUresult r = g_encode(map, dt, 2, const_cast<void*>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? G2_OK : G2_ERR_ARG;
}

}  // namespace g2

extern "C" int g2_abi_version(void) { return G2_ABI_VERSION; }

extern "C" const char* g2_status_string(int status) {
  switch (status) {
    case G2_OK: return "ok";
    case G2_ERR_ARG: return "invalid argument";
    case G2_ERR_CUDA: return "CUDA runtime error";
    case G2_ERR_UNSUPPORTED: return "unsupported device or feature";
    case G2_ERR_TOO_LARGE: return "size exceeds a kernel limit";
    default: return "unknown status";
  }
}

extern "C" int g2_device_info(int device, int32_t* sm_count, int32_t* cc_major, int32_t* cc_minor) {
  if (!sm_count || !cc_major || !cc_minor) return G2_ERR_ARG;
  int n = 0, ma = 0, mi = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return G2_ERR_CUDA;
  if (cudaDeviceGetAttribute(&ma, cudaDevAttrComputeCapabilityMajor, device) != cudaSuccess) return G2_ERR_CUDA;
  if (cudaDeviceGetAttribute(&mi, cudaDevAttrComputeCapabilityMinor, device) != cudaSuccess) return G2_ERR_CUDA;
  *sm_count = n;
  *cc_major = ma;
  *cc_minor = mi;
  return G2_OK;
}

// Longest-processing-time list schedule of a launch's items over the
// persistent workers (host code: no device is touched).  Items in descending
// cost (ties in index order) go one by one to the least-loaded worker (ties
// to the lower worker index); each worker then keeps its items in index
// order, and worker w's k-th item lands in slot w + k * workers -- the slots
// the kernels read.  slot_out[i] is item i's slot; *n_slots the length of the
// slot list (workers times the longest worker list).
extern "C" int g2_balance_lpt(const double* cost, int64_t n, int32_t workers, int64_t* slot_out,
                              int64_t* n_slots) {
  if (!cost || !slot_out || !n_slots || n < 0 || workers <= 0) return G2_ERR_ARG;
  for (int64_t i = 0; i < n; ++i)
    if (!(cost[i] >= 0.0)) return G2_ERR_ARG;  // also rejects NaN
  std::vector<int64_t> order(static_cast<size_t>(n));
  std::iota(order.begin(), order.end(), int64_t(0));
  std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return cost[a] > cost[b]; });
  using Slot = std::pair<double, int32_t>;
  std::priority_queue<Slot, std::vector<Slot>, std::greater<Slot>> heap;
  for (int32_t w = 0; w < workers; ++w) heap.push(Slot(0.0, w));
  std::vector<int32_t> owner(static_cast<size_t>(n));
  for (int64_t i : order) {
    Slot s = heap.top();
    heap.pop();
    owner[static_cast<size_t>(i)] = s.second;
    heap.push(Slot(s.first + cost[i], s.second));
  }
  std::vector<int64_t> next(static_cast<size_t>(workers), 0);
  int64_t longest = 0;
  for (int64_t i = 0; i < n; ++i) {  // index order within each worker
    const int32_t w = owner[static_cast<size_t>(i)];
    slot_out[i] = w + next[static_cast<size_t>(w)] * workers;
    longest = std::max(longest, ++next[static_cast<size_t>(w)]);
  }
  *n_slots = longest * workers;
  return G2_OK;
}

// Host-to-device copy of a column window of many rows: the frames of a stack
// cropped to the q-mask's bounding columns, so that only those bytes cross
// the host link.  One cudaMemcpy2DAsync (the copy engines walk the rows).
extern "C" int g2_copy_cols_h2d(void* dst_dev, const void* src_host, int64_t src_pitch, int64_t col0, int64_t width,
                                int64_t rows, void* stream) {
  if (!dst_dev || !src_host || src_pitch <= 0 || col0 < 0 || width <= 0 || col0 + width > src_pitch || rows < 0)
    return G2_ERR_ARG;
  if (rows == 0) return G2_OK;
  const cudaError_t e = cudaMemcpy2DAsync(dst_dev, static_cast<size_t>(width),
                                          static_cast<const char*>(src_host) + col0, static_cast<size_t>(src_pitch),
                                          static_cast<size_t>(width), static_cast<size_t>(rows),
                                          cudaMemcpyHostToDevice, g2::as_stream(stream));
  return e == cudaSuccess ? G2_OK : G2_ERR_CUDA;
}
