// Host-side helpers shared by the C-ABI translation units (not part of the ABI).
#pragma once
#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>
#include "../../include/dynamix_g2.h"

namespace g2 {

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline bool aligned(const void* p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

// Map the last CUDA error (launch configuration etc.) to a status code.
inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? G2_OK : G2_ERR_CUDA;
}

// Current device's SM count (cached per device).
int sm_count_current();

// Encode a 2-D tiled tensor map over a row-major [rows][cols] matrix of
// 2-byte (fp16) or 1-byte (e4m3, as uint8) elements with a (box_cols x
// box_rows) box, 128-byte swizzle, zero fill outside.
int encode_tmap_2d(CUtensorMap* map, const void* base, int elem_bytes, uint64_t cols, uint64_t rows,
                   uint32_t box_cols, uint32_t box_rows);

}  // namespace g2
