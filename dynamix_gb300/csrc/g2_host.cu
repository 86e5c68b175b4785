// Host utilities of the C ABI: status strings, device queries, tensor maps.
#include <cstring>
#include <mutex>
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
