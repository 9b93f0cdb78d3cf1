// Stable LSD radix sort of 64-bit keys with optional 64-bit payloads.
//
// One pass per 8-bit digit, three launches per pass:
//   radix_hist     per tile of kTile keys, the count of each digit value
//                  (per-warp shared counters, then summed), written
//                  digit-major (hist[1 + d * ntiles + tile]);
//   scan           inclusive prefix sum of the histogram, so hist[d * ntiles
//                  + tile] becomes the global output offset of the tile's
//                  first key with digit d (digits in order, tiles in order:
//                  stability across tiles);
//   radix_scatter  each tile ranks its keys stably (warp match on the digit,
//                  per-warp running counts, warps in order), stages the tile
//                  in shared memory in digit order and writes each digit run
//                  to its global offset, so the stores of one run are
//                  contiguous.
// Traffic per pass and key: 8 B read (histogram) + 16 B read + 16 B written
// (keys and payloads), plus 8 B x 256 / kTile of histogram.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;                       // keys per thread
constexpr int kTile = kThreads * kItems;        // 2048 keys per tile
constexpr int kWarps = kThreads / 32;
constexpr int kWarpItems = kTile / kWarps;      // 256 consecutive keys per warp

__device__ __forceinline__ int digit_of(uint64_t k, int shift, uint32_t mask) {
  return (int)((k >> shift) & mask);
}

// Per-warp shared counters (plain shared atomics: a warp's lanes collide only
// when their digits are equal), summed over the warps at the end.  The keys
// of one thread are loaded together (kItems loads in flight).
__global__ void __launch_bounds__(kThreads) radix_hist(int64_t n, const uint64_t* __restrict__ keys, int shift,
                                                       uint32_t mask, int64_t ntiles, int64_t* __restrict__ hist) {
  __shared__ int cnt[kWarps][256];
  for (int i = threadIdx.x; i < kWarps * 256; i += kThreads) (&cnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t t = blockIdx.x, base = t * kTile;
  const int w = threadIdx.x >> 5;
  uint64_t k[kItems];
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const int64_t e = base + j * kThreads + threadIdx.x;
    k[j] = e < n ? __ldg(keys + e) : 0;
  }
#pragma unroll
  for (int j = 0; j < kItems; ++j)
    if (base + j * kThreads + threadIdx.x < n) atomicAdd(&cnt[w][digit_of(k[j], shift, mask)], 1);
  __syncthreads();
  for (int d = threadIdx.x; d < 256; d += kThreads) {
    int s = 0;
#pragma unroll
    for (int i = 0; i < kWarps; ++i) s += cnt[i][d];
    hist[1 + (int64_t)d * ntiles + t] = s;
  }
  if (t == 0 && threadIdx.x == 0) hist[0] = 0;
}

// exclusive scan of 256 ints held one per thread (kThreads == 256)
__device__ __forceinline__ int block_exclusive_scan256(int v, int* warp_tot) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  int off = 0;
  for (int i = 0; i < w; ++i) off += warp_tot[i];
  return off + x - v;
}

__global__ void __launch_bounds__(kThreads) radix_scatter(int64_t n, const uint64_t* __restrict__ kin,
                                                          const uint64_t* __restrict__ vin, uint64_t* __restrict__ kout,
                                                          uint64_t* __restrict__ vout, int shift, uint32_t mask,
                                                          int64_t ntiles, const int64_t* __restrict__ hist) {
  __shared__ uint64_t sk[kTile];
  __shared__ uint64_t sv[kTile];
  __shared__ int wcnt[kWarps][256];
  __shared__ int dstart[256];
  __shared__ int64_t gbase[256];
  __shared__ int wtot[kWarps];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int i = threadIdx.x; i < kWarps * 256; i += kThreads) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int64_t t = blockIdx.x, base = t * kTile;
  const bool has_v = vin != nullptr;
  uint64_t k[kItems], v[kItems];
  int r[kItems];
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const int64_t e = base + w * kWarpItems + j * 32 + lane;
    k[j] = e < n ? kin[e] : 0;
    v[j] = (e < n && has_v) ? vin[e] : 0;
  }
  // stable ranks: keys in warp-item order, warps in order
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const int64_t e = base + w * kWarpItems + j * 32 + lane;
    const bool valid = e < n;
    const unsigned act = __ballot_sync(0xffffffffu, valid);
    int prior = 0, d = 0;
    unsigned peers = 0;
    if (valid) {
      d = digit_of(k[j], shift, mask);
      peers = __match_any_sync(act, d);
      prior = wcnt[w][d];
      r[j] = prior + __popc(peers & ((1u << lane) - 1u));
    }
    __syncwarp();
    if (valid && lane == __ffs(peers) - 1) wcnt[w][d] = prior + __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  {
    const int d = threadIdx.x;  // kThreads == 256 digits
    int tot = 0;
    for (int i = 0; i < kWarps; ++i) {
      const int c = wcnt[i][d];
      wcnt[i][d] = tot;
      tot += c;
    }
    dstart[d] = block_exclusive_scan256(tot, wtot);
    gbase[d] = hist[(int64_t)d * ntiles + t];
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < kItems; ++j) {
    const int64_t e = base + w * kWarpItems + j * 32 + lane;
    if (e < n) {
      const int d = digit_of(k[j], shift, mask);
      const int p = dstart[d] + wcnt[w][d] + r[j];
      sk[p] = k[j];
      if (has_v) sv[p] = v[j];
    }
  }
  __syncthreads();
  const int cnt = (int)(n - base < kTile ? n - base : kTile);
  for (int i = threadIdx.x; i < cnt; i += kThreads) {
    const uint64_t key = sk[i];
    const int d = digit_of(key, shift, mask);
    const int64_t o = gbase[d] + (i - dstart[d]);
    kout[o] = key;
    if (has_v) vout[o] = sv[i];
  }
}

}  // namespace

int64_t radix_scratch_bytes(int64_t n) {
  const int64_t ntiles = (n + kTile - 1) / kTile;
  const int64_t h = 1 + 256 * (ntiles < 1 ? 1 : ntiles);
  const int64_t hb = (h * (int64_t)sizeof(int64_t) + 255) / 256 * 256;
  return hb + scan_scratch_bytes(h);
}

cudaError_t radix_sort_u64(int64_t n, uint64_t* keys, uint64_t* vals, uint64_t* keys_alt, uint64_t* vals_alt,
                           int begin_bit, int end_bit, void* scratch, cudaStream_t s, bool* in_alt) {
  *in_alt = false;
  if (n <= 1 || end_bit <= begin_bit) return cudaSuccess;
  const int64_t ntiles = (n + kTile - 1) / kTile;
  const int64_t h = 1 + 256 * ntiles;
  int64_t* hist = reinterpret_cast<int64_t*>(scratch);
  void* scan_scratch = static_cast<char*>(scratch) + (h * (int64_t)sizeof(int64_t) + 255) / 256 * 256;
  uint64_t *ki = keys, *vi = vals, *ko = keys_alt, *vo = vals_alt;
  for (int shift = begin_bit; shift < end_bit; shift += 8) {
    const int bits = end_bit - shift < 8 ? end_bit - shift : 8;
    const uint32_t mask = (1u << bits) - 1u;
    radix_hist<<<(unsigned)ntiles, kThreads, 0, s>>>(n, ki, shift, mask, ntiles, hist);
    cudaError_t e = inclusive_scan_i64(hist, h, scan_scratch, s);
    if (e != cudaSuccess) return e;
    radix_scatter<<<(unsigned)ntiles, kThreads, 0, s>>>(n, ki, vals ? vi : nullptr, ko, vals ? vo : nullptr, shift, mask,
                                                        ntiles, hist);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint64_t* tk = ki; ki = ko; ko = tk;
    uint64_t* tv = vi; vi = vo; vo = tv;
    *in_alt = !*in_alt;
  }
  return cudaSuccess;
}

}  // namespace sg

using namespace sg;

extern "C" int64_t sg_radix_scratch_bytes(int64_t n) { return n < 0 ? -1 : radix_scratch_bytes(n); }

extern "C" int sg_radix_sort_u64(int64_t n, uint64_t* keys, uint64_t* vals, uint64_t* keys_alt, uint64_t* vals_alt,
                                 int begin_bit, int end_bit, void* scratch, int* result_in_alt, void* stream) {
  if (n < 0 || begin_bit < 0 || end_bit > 64 || begin_bit > end_bit || !result_in_alt) return SG_ERR_ARG;
  if (n > 1 && (!keys || !keys_alt || !scratch || (vals && !vals_alt))) return SG_ERR_ARG;
  bool alt = false;
  const cudaError_t e = radix_sort_u64(n, keys, vals, keys_alt, vals_alt, begin_bit, end_bit, scratch,
                                       as_stream(stream), &alt);
  *result_in_alt = alt ? 1 : 0;
  return e == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}
