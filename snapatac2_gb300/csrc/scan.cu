// Device-wide inclusive scan of int64 (reduce -> scan of tile sums -> add).
#include "common.cuh"
#include "internal.h"

namespace sg {

namespace {

__global__ void __launch_bounds__(kScanBlock) tile_reduce(const int64_t* __restrict__ d, int64_t n,
                                                           int64_t* __restrict__ sums) {
  __shared__ long long ws[kScanBlock / 32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  long long s = 0;
#pragma unroll
  for (int j = 0; j < kScanItems; ++j) {
    int64_t i = base + (int64_t)j * kScanBlock + threadIdx.x;
    if (i < n) s += d[i];
  }
  s = block_sum_ll<kScanBlock>(s, ws);
  if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

// Exclusive scan of the tile sums by a single block.
__global__ void __launch_bounds__(1024) sums_scan(int64_t* sums, int64_t nt) {
  __shared__ long long carry;
  __shared__ long long ws[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int64_t b = 0; b < nt; b += 1024) {
    int64_t i = b + threadIdx.x;
    long long v = i < nt ? sums[i] : 0;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
      long long t = ws[lane];
      for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      ws[lane] = t;
    }
    __syncthreads();
    long long excl = carry + (wid ? ws[wid - 1] : 0) + x - v;
    if (i < nt) sums[i] = excl;
    __syncthreads();
    if (threadIdx.x == 0) carry += ws[31];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanBlock) tile_scan(int64_t* __restrict__ d, int64_t n,
                                                         const int64_t* __restrict__ sums) {
  __shared__ long long ws[kScanBlock / 32];
  __shared__ long long carry;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kScanTile;
  if (threadIdx.x == 0) carry = sums[blockIdx.x];
  __syncthreads();
  for (int j = 0; j < kScanItems; ++j) {
    int64_t i = base + (int64_t)j * kScanBlock + threadIdx.x;
    long long v = i < n ? d[i] : 0;
    long long x = v;
    for (int o = 1; o < 32; o <<= 1) {
      long long y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
      long long t = lane < kScanBlock / 32 ? ws[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      if (lane < kScanBlock / 32) ws[lane] = t;
    }
    __syncthreads();
    long long incl = carry + (wid ? ws[wid - 1] : 0) + x;
    if (i < n) d[i] = incl;
    __syncthreads();
    if (threadIdx.x == 0) carry += ws[kScanBlock / 32 - 1];
    __syncthreads();
  }
}

}  // namespace

int64_t scan_scratch_bytes(int64_t n) {
  int64_t nt = (n + kScanTile - 1) / kScanTile;
  return (nt < 1 ? 1 : nt) * (int64_t)sizeof(int64_t);
}

cudaError_t inclusive_scan_i64(int64_t* data, int64_t n, void* scratch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  int64_t nt = (n + kScanTile - 1) / kScanTile;
  int64_t* sums = reinterpret_cast<int64_t*>(scratch);
  tile_reduce<<<(unsigned)nt, kScanBlock, 0, s>>>(data, n, sums);
  sums_scan<<<1, 1024, 0, s>>>(sums, nt);
  tile_scan<<<(unsigned)nt, kScanBlock, 0, s>>>(data, n, sums);
  return cudaGetLastError();
}

}  // namespace sg
