// Gather ceiling of the Gram SpMM: the row gathers of one SpMM pass and
// nothing else.  For every nonzero e the row table[idx[e]] (block values,
// 16-byte vectors, LPN lanes per row as in the SpMM kernels) is loaded and
// folded into a register; no segmented reduction, no scaling, no output rows.
// Its time over a matrix's own index stream is the floor the SpMM pass can
// reach with this memory access pattern (one L1/L2 line per gathered row at
// block 8 FP32), which the benchmark reports beside the HBM roofline.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

template <typename T, int B>
__global__ void __launch_bounds__(256) gather_ceiling_kernel(int64_t nnz, const int32_t* __restrict__ idx,
                                                             const T* __restrict__ table, float* __restrict__ sink) {
  using VT = typename V16<T>::type;
  constexpr int LPN = B / V16<T>::n;
  constexpr int NPS = 32 / LPN;  // nonzeros per warp step
  constexpr int U = 4;
  const int lane = threadIdx.x & 31, slot = lane / LPN, sub = lane % LPN;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  VT acc = V16<T>::zero();
  for (int64_t base = gw * NPS * U; base < nnz; base += nw * NPS * U) {
    int c[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int64_t e = base + u * NPS + slot;
      c[u] = e < nnz ? __ldg(idx + e) : -1;
    }
#pragma unroll
    for (int u = 0; u < U; ++u)
      if (c[u] >= 0) V16<T>::add(acc, __ldg(reinterpret_cast<const VT*>(table + (int64_t)c[u] * B) + sub));
  }
  const T* a = reinterpret_cast<const T*>(&acc);
  T s = T(0);
#pragma unroll
  for (int q = 0; q < V16<T>::n; ++q) s += a[q];
  if (s == T(-1.2345e-30)) sink[0] = (float)s;  // keeps the loads; never true for the tables used
}

int sms_diag() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

template <typename T>
int launch_gather(int block, int64_t nnz, const int32_t* idx, const void* table, float* sink, cudaStream_t s) {
  const int grid = 8 * sms_diag();
  const T* t = static_cast<const T*>(table);
  switch (block) {
    case 4: gather_ceiling_kernel<T, 4><<<grid, 256, 0, s>>>(nnz, idx, t, sink); break;
    case 8: gather_ceiling_kernel<T, 8><<<grid, 256, 0, s>>>(nnz, idx, t, sink); break;
    case 16: gather_ceiling_kernel<T, 16><<<grid, 256, 0, s>>>(nnz, idx, t, sink); break;
    case 32: gather_ceiling_kernel<T, 32><<<grid, 256, 0, s>>>(nnz, idx, t, sink); break;
    default: return SG_ERR_ARG;
  }
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_gather_ceiling(int dtype, int block, int64_t nnz, const int32_t* idx, const void* table,
                                 float* sink, void* stream) {
  if (nnz < 0 || !table || !sink || (nnz > 0 && !idx)) return SG_ERR_ARG;
  if (nnz == 0) return SG_OK;
  if (dtype == 0) return launch_gather<float>(block, nnz, idx, table, sink, as_stream(stream));
  if (dtype == 1) return launch_gather<double>(block, nnz, idx, table, sink, as_stream(stream));
  return SG_ERR_ARG;
}
