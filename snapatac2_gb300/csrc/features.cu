// Per-feature (column) sums of a cell-by-feature CSR matrix: the `count`
// vector of select_features (snapatac2-python/python/snapatac2/preprocessing/
// _basic.py:1053-1056, which adds X.sum(axis=0) over 2000-row chunks into an
// FP64 vector).
//
// Count values (uint32, or the implicit 1 of a binary pattern) are summed in
// uint64 with atomics: integer addition is exact and associative, so the
// result is the same whatever the order of the atomics, and its conversion
// to FP64 equals the reference's FP64 sum (every partial sum stays below
// 2^53).  FP32 values are summed in FP64 with atomics (exact when the values
// are integers, as count matrices are).  Column indices outside [0, m) set
// status SG_ERR_ARG with the first offending entry and are not counted.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

template <int KIND>  // 0 = binary, 1 = uint32 counts, 2 = float32 values
__global__ void col_count_kernel(int64_t nnz, int64_t m, const int32_t* __restrict__ idx,
                                 const uint32_t* __restrict__ cnt, const float* __restrict__ val,
                                 unsigned long long* __restrict__ acc_u, double* __restrict__ acc_f,
                                 int* status, unsigned long long* bad) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
    const int c = idx[e];
    if (c < 0 || c >= m) {
      report_error(status, bad, SG_ERR_ARG, (unsigned long long)e);
      continue;
    }
    if (KIND == 0) atomicAdd(acc_u + c, 1ull);
    else if (KIND == 1) atomicAdd(acc_u + c, (unsigned long long)cnt[e]);
    else atomicAdd(acc_f + c, (double)val[e]);
  }
}

__global__ void u64_to_f64(int64_t m, const unsigned long long* __restrict__ in, double* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x)
    out[j] = (double)in[j];
}

int sms_features() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_col_counts(int64_t nnz, int64_t m, const int32_t* indices, const uint32_t* counts,
                             const float* values, double* out, unsigned long long* scratch, int* status,
                             unsigned long long* bad, void* stream) {
  if (nnz < 0 || m <= 0 || !out || !status || (nnz > 0 && !indices) || (counts && values) ||
      (!values && !scratch))
    return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int grid = grid_for(nnz > 0 ? nnz : 1, 256, 16 * sms_features());
  if (values) {
    if (cudaMemsetAsync(out, 0, (size_t)m * sizeof(double), s) != cudaSuccess) return SG_ERR_CUDA;
    if (nnz > 0)
      col_count_kernel<2><<<grid, 256, 0, s>>>(nnz, m, indices, nullptr, values, nullptr, out, status, bad);
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  if (cudaMemsetAsync(scratch, 0, (size_t)m * sizeof(unsigned long long), s) != cudaSuccess) return SG_ERR_CUDA;
  if (nnz > 0) {
    if (counts) col_count_kernel<1><<<grid, 256, 0, s>>>(nnz, m, indices, counts, nullptr, scratch, nullptr, status, bad);
    else col_count_kernel<0><<<grid, 256, 0, s>>>(nnz, m, indices, nullptr, nullptr, scratch, nullptr, status, bad);
    SG_CHECK_LAUNCH();
  }
  u64_to_f64<<<grid_for(m, 256, 16 * sms_features()), 256, 0, s>>>(m, scratch, out);
  SG_CHECK_LAUNCH();
  return SG_OK;
}
