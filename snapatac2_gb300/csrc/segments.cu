// Row, segment and chunk steps around the main kernels (gene matrix,
// Nyström, import), so that these run in this library rather than as
// framework tensor operations:
//   sg_csr_row_ptr,      rows of a CSR, in a given order (Nyström landmarks):
//   sg_csr_copy_rows     the new row pointer, then the copy;
//   sg_gather_bytes      byte segments into one contiguous buffer (barcodes);
//   sg_gene_max          per row, the maximum count over the regions of each
//                        gene (GeneCount::get_values,
//                        snapatac2-core/src/feature_count/counter.rs:270-283):
//                        (row, gene) keys radix-sorted with their counts,
//                        runs reduced by maximum;
//   sg_nystrom_rescale   the per-chunk rescaling of nystrom's embedded Python
//                        (snapatac2-python/src/embedding.rs:222-229): t = Σ_chunk q ⊙ λ,
//                        d = q t, d <= 0 -> the chunk's smallest positive d,
//                        q /= sqrt(d); one CTA per chunk, a warp per row.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kThreads = 256;

__global__ void row_lengths(int64_t k, const int64_t* __restrict__ rows, const int64_t* __restrict__ indptr,
                            int64_t* __restrict__ out_ptr) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < k; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = rows[i];
    out_ptr[i + 1] = indptr[r + 1] - indptr[r];
    if (i == 0) out_ptr[0] = 0;
  }
}

// warp per selected row: contiguous copy of its indices (and values)
__global__ void copy_rows(int64_t k, const int64_t* __restrict__ rows, const int64_t* __restrict__ indptr,
                          const int32_t* __restrict__ idx, const float* __restrict__ val,
                          const int64_t* __restrict__ out_ptr, int32_t* __restrict__ oidx, float* __restrict__ oval) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < k; i += nw) {
    const int64_t r = rows[i], s = indptr[r], n = indptr[r + 1] - s, d = out_ptr[i];
    for (int64_t j = lane; j < n; j += 32) {
      oidx[d + j] = idx[s + j];
      if (val) oval[d + j] = val[s + j];
    }
  }
}

__global__ void copy_bytes(int64_t k, const int64_t* __restrict__ off, const int32_t* __restrict__ len,
                           const int64_t* __restrict__ dst_off, const uint8_t* __restrict__ src,
                           uint8_t* __restrict__ dst) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < k; i += nw)
    for (int j = lane; j < len[i]; j += 32) dst[dst_off[i] + j] = src[off[i] + j];
}

// keys (row << 32 | gene) and counts of every region entry
__global__ void gene_keys(int64_t n, const int64_t* __restrict__ indptr, const int32_t* __restrict__ region,
                          const uint32_t* __restrict__ cnt, const int32_t* __restrict__ region_gene,
                          uint64_t* __restrict__ keys, uint64_t* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < n; r += nw)
    for (int64_t e = indptr[r] + lane; e < indptr[r + 1]; e += 32) {
      keys[e] = ((uint64_t)r << 32) | (uint32_t)region_gene[region[e]];
      vals[e] = cnt[e];
    }
}

__global__ void run_heads(int64_t nnz, const uint64_t* __restrict__ keys, int64_t* __restrict__ head) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x)
    head[e] = e == 0 || keys[e] != keys[e - 1];
}

// run u = head_scan[e] - 1: its key and the maximum count (order-free)
__global__ void run_max(int64_t nnz, const uint64_t* __restrict__ keys, const uint64_t* __restrict__ vals,
                        const int64_t* __restrict__ head_scan, uint64_t* __restrict__ ukey,
                        unsigned long long* __restrict__ umax) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t u = head_scan[e] - 1;
    if (e == 0 || keys[e] != keys[e - 1]) ukey[u] = keys[e];
    atomicMax(umax + u, (unsigned long long)vals[e]);
  }
}

__global__ void run_out(int64_t U, const uint64_t* __restrict__ ukey, const unsigned long long* __restrict__ umax,
                        int32_t* __restrict__ oidx, int32_t* __restrict__ oval) {
  for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < U; u += (int64_t)gridDim.x * blockDim.x) {
    oidx[u] = (int32_t)(ukey[u] & 0xffffffffu);
    oval[u] = (int32_t)(uint32_t)umax[u];
  }
}

// out_ptr[r] = first run whose row is >= r (runs sorted by row): a row pointer
__global__ void row_bounds(int64_t n, int64_t U, const uint64_t* __restrict__ ukey, int64_t* __restrict__ out_ptr) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r <= n; r += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = U;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if ((int64_t)(ukey[mid] >> 32) < r) lo = mid + 1;
      else hi = mid;
    }
    out_ptr[r] = lo;
  }
}

// One CTA per chunk of rows, a warp per row and the lanes across its k
// columns (coalesced row reads): t = λ ⊙ Σ_chunk rows, d_i = q_i · t,
// d <= 0 -> the chunk's smallest positive d, q_i /= sqrt(d_i).  Fixed
// summation orders (warp-strided partial sums, warps in order; lane-strided
// products, then a fixed butterfly).  A chunk with some d <= 0 and none
// positive is an error (the reference's np.min of an empty array raises):
// SG_ERR_NUMERIC, bad = the chunk's first row.
constexpr int kWarpsR = kThreads / 32;
constexpr int kMaxCols = 256;

__device__ __forceinline__ double row_dot(const double* __restrict__ q, int64_t r, int k, int lane,
                                          const double* __restrict__ t) {
  double v = 0.0;
  for (int c = lane; c < k; c += 32) v += q[r * k + c] * t[c];
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__global__ void __launch_bounds__(kThreads) nystrom_rescale_kernel(int64_t n, int k, double* __restrict__ q,
                                                                   const double* __restrict__ evals, int64_t chunk,
                                                                   int* status, unsigned long long* bad) {
  __shared__ double part[kWarpsR][kMaxCols];
  __shared__ double t[kMaxCols];
  __shared__ double wmin[kWarpsR];
  __shared__ int wneg[kWarpsR];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t r0 = blockIdx.x * chunk;
  const int64_t r1 = r0 + chunk < n ? r0 + chunk : n;
  for (int c = lane; c < k; c += 32) {
    double s = 0.0;
    for (int64_t r = r0 + w; r < r1; r += kWarpsR) s += q[r * k + c];
    part[w][c] = s;
  }
  __syncthreads();
  for (int c = threadIdx.x; c < k; c += kThreads) {
    double s = 0.0;
    for (int i = 0; i < kWarpsR; ++i) s += part[i][c];
    t[c] = s * evals[c];
  }
  __syncthreads();
  double mn = INFINITY;
  int neg = 0;
  for (int64_t r = r0 + w; r < r1; r += kWarpsR) {
    const double d = row_dot(q, r, k, lane, t);
    if (d > 0.0) mn = fmin(mn, d);
    else neg = 1;
  }
  if (lane == 0) { wmin[w] = mn; wneg[w] = neg; }
  __syncthreads();
  double dmin = INFINITY;
  int anyneg = 0;
  for (int i = 0; i < kWarpsR; ++i) { dmin = fmin(dmin, wmin[i]); anyneg |= wneg[i]; }
  if (anyneg && dmin == INFINITY) {
    if (threadIdx.x == 0) report_error(status, bad, SG_ERR_NUMERIC, (unsigned long long)r0);
    return;
  }
  for (int64_t r = r0 + w; r < r1; r += kWarpsR) {
    double d = row_dot(q, r, k, lane, t);
    if (!(d > 0.0)) d = dmin;
    const double sd = sqrt(d);
    for (int c = lane; c < k; c += 32) q[r * k + c] /= sd;
  }
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_csr_row_ptr(int64_t k, const int64_t* rows, const int64_t* indptr, int64_t* out_ptr,
                              void* scan_scratch, void* stream) {
  if (k < 0 || (k > 0 && (!rows || !indptr || !out_ptr || !scan_scratch))) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (k == 0) return cudaMemsetAsync(out_ptr, 0, 8, s) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
  row_lengths<<<grid_for(k, kThreads), kThreads, 0, s>>>(k, rows, indptr, out_ptr);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(out_ptr + 1, k, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}

extern "C" int sg_csr_copy_rows(int64_t k, const int64_t* rows, const int64_t* indptr, const int32_t* indices,
                                const float* values, const int64_t* out_ptr, int32_t* out_idx, float* out_val,
                                void* stream) {
  if (k < 0 || (k > 0 && (!rows || !indptr || !indices || !out_ptr || !out_idx))) return SG_ERR_ARG;
  if (values && !out_val) return SG_ERR_ARG;
  if (k == 0) return SG_OK;
  copy_rows<<<grid_for(k * 32, kThreads, 8 * 152 * 8), kThreads, 0, as_stream(stream)>>>(k, rows, indptr, indices,
                                                                                         values, out_ptr, out_idx,
                                                                                         out_val);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_gather_bytes(int64_t k, const int64_t* off, const int32_t* len, const int64_t* dst_off,
                               const uint8_t* src, uint8_t* dst, void* stream) {
  if (k < 0 || (k > 0 && (!off || !len || !dst_off || !src || !dst))) return SG_ERR_ARG;
  if (k == 0) return SG_OK;
  copy_bytes<<<grid_for(k * 32, kThreads, 8 * 152 * 8), kThreads, 0, as_stream(stream)>>>(k, off, len, dst_off, src,
                                                                                          dst);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int64_t sg_gene_max_scratch_bytes(int64_t nnz) {
  if (nnz < 0) return -1;
  const int64_t n8 = ((nnz < 1 ? 1 : nnz) * 8 + 255) / 256 * 256;
  return 5 * n8 + (radix_scratch_bytes(nnz < 1 ? 1 : nnz) + 255) / 256 * 256 + scan_scratch_bytes(nnz + 1);
}

// out_ptr[n + 1]; out_idx / out_val need nnz entries (at most nnz runs);
// *n_out (host) = number of (row, gene) entries.  Synchronises the stream.
extern "C" int sg_gene_max(int64_t n, const int64_t* indptr, const int32_t* region, const uint32_t* counts,
                           const int32_t* region_gene, int64_t nnz, void* scratch, int64_t scratch_bytes,
                           int64_t* out_ptr, int32_t* out_idx, int32_t* out_val, int64_t* n_out, void* stream) {
  if (n < 0 || nnz < 0 || n >= (int64_t(1) << 31) || !n_out || !out_ptr) return SG_ERR_ARG;
  if (nnz > 0 && (!indptr || !region || !counts || !region_gene || !scratch || !out_idx || !out_val))
    return SG_ERR_ARG;
  if (scratch_bytes < sg_gene_max_scratch_bytes(nnz)) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  *n_out = 0;
  if (nnz == 0) {
    if (cudaMemsetAsync(out_ptr, 0, (n + 1) * 8, s) != cudaSuccess) return SG_ERR_CUDA;
    return cudaStreamSynchronize(s) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
  }
  const int64_t n8 = (nnz * 8 + 255) / 256 * 256;
  char* w = static_cast<char*>(scratch);
  uint64_t* k0 = reinterpret_cast<uint64_t*>(w);
  uint64_t* v0 = reinterpret_cast<uint64_t*>(w + n8);
  uint64_t* k1 = reinterpret_cast<uint64_t*>(w + 2 * n8);
  uint64_t* v1 = reinterpret_cast<uint64_t*>(w + 3 * n8);
  int64_t* head = reinterpret_cast<int64_t*>(w + 4 * n8);
  void* rscr = w + 5 * n8;
  void* sscr = w + 5 * n8 + (radix_scratch_bytes(nnz) + 255) / 256 * 256;
  const int g = grid_for(n * 32, kThreads, 8 * 152 * 8);
  gene_keys<<<g, kThreads, 0, s>>>(n, indptr, region, counts, region_gene, k0, v0);
  SG_CHECK_LAUNCH();
  int rbits = 1;
  while (rbits < 31 && ((int64_t)1 << rbits) < n) ++rbits;
  bool alt = false;
  if (radix_sort_u64(nnz, k0, v0, k1, v1, 0, 32 + rbits, rscr, s, &alt) != cudaSuccess) return SG_ERR_CUDA;
  const uint64_t* keys = alt ? k1 : k0;
  const uint64_t* vals = alt ? v1 : v0;
  run_heads<<<grid_for(nnz, kThreads), kThreads, 0, s>>>(nnz, keys, head);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(head, nnz, sscr, s) != cudaSuccess) return SG_ERR_CUDA;
  int64_t U = 0;
  if (cudaMemcpyAsync(&U, head + nnz - 1, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) return SG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SG_ERR_CUDA;
  uint64_t* ukey = alt ? k0 : k1;  // the free pair
  unsigned long long* umax = reinterpret_cast<unsigned long long*>(alt ? v0 : v1);
  if (cudaMemsetAsync(umax, 0, U * 8, s) != cudaSuccess) return SG_ERR_CUDA;
  run_max<<<grid_for(nnz, kThreads), kThreads, 0, s>>>(nnz, keys, vals, head, ukey, umax);
  SG_CHECK_LAUNCH();
  run_out<<<grid_for(U, kThreads), kThreads, 0, s>>>(U, ukey, umax, out_idx, out_val);
  row_bounds<<<grid_for(n + 1, kThreads), kThreads, 0, s>>>(n, U, ukey, out_ptr);
  SG_CHECK_LAUNCH();
  if (cudaStreamSynchronize(s) != cudaSuccess) return SG_ERR_CUDA;
  *n_out = U;
  return SG_OK;
}

extern "C" int sg_nystrom_rescale(int64_t n, int k, double* q, const double* evals, int64_t chunk, int* status,
                                  unsigned long long* bad, void* stream) {
  if (n < 0 || k < 1 || k > kMaxCols || chunk < 1 || (n > 0 && (!q || !evals || !status))) return SG_ERR_ARG;
  if (n == 0) return SG_OK;
  const int64_t nchunks = (n + chunk - 1) / chunk;
  if (nchunks > 0x7fffffff) return SG_ERR_ARG;
  nystrom_rescale_kernel<<<(unsigned)nchunks, kThreads, 0, as_stream(stream)>>>(n, k, q, evals, chunk, status,
                                                                                  bad);
  SG_CHECK_LAUNCH();
  return SG_OK;
}
