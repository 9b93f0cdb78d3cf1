// Internal (C++ linkage) helpers shared between translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanBlock * kScanItems;

// In-place inclusive prefix sum of n int64 values.  `scratch` needs
// scan_scratch_bytes(n) bytes.  Deterministic.
cudaError_t inclusive_scan_i64(int64_t* data, int64_t n, void* scratch, cudaStream_t s);
int64_t scan_scratch_bytes(int64_t n);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int grid_for(int64_t n, int block, int max_blocks = 1 << 20) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

}  // namespace sg
