// Aggregation of an existing cell-by-feature matrix by regions: the use_x
// path of the peak and gene matrices, which replaces
//   create_peak_matrix / create_gene_matrix with use_x
//   (snapatac2-core/src/feature_count/matrix.rs:121-128,211-218):
//   read_chrom_values().aggregate_by(counter) (data_iter.rs:866-891), where
//   each entry (feature interval j, value v) of a cell's row adds v to every
//   region overlapping interval j (RegionCounter::insert, counter.rs:95-106).
//
// With M the feature -> region overlap map (CSR, built on the host from the
// intervals), the result is the sparse product X·M.  Every entry of X is
// expanded into (cell, region, value) records keyed (cell << rbits) | region,
// the keys are radix-sorted (stable, so equal keys keep X's column order),
// equal keys are summed in that order and each cell's row comes out sorted by
// region, as the reference's per-row BTreeMap emits it.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

// expanded records of row r: sum of |M[idx]| over its entries
__global__ void agg_count_kernel(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                 const int64_t* __restrict__ fptr, int64_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w; r < n; r += nw) {
    int64_t c = 0;
    for (int64_t e = ptr[r] + lane; e < ptr[r + 1]; e += 32) {
      const int j = idx[e];
      c += fptr[j + 1] - fptr[j];
    }
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[r + 1] = c;
    if (r == 0 && lane == 0) cnt[0] = 0;
  }
}

// record t of row r at eoff[r] + (its rank): key = (r << rbits) | region,
// value bits = the entry's value (uint32 widened, or the FP64 bits)
__global__ void agg_expand_kernel(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                                  const void* __restrict__ val, int dtype, const int64_t* __restrict__ fptr,
                                  const int32_t* __restrict__ freg, const int64_t* __restrict__ eoff, int rbits,
                                  uint64_t* __restrict__ keys, uint64_t* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w; r < n; r += nw) {
    int64_t o = eoff[r];
    for (int64_t e0 = ptr[r]; e0 < ptr[r + 1]; e0 += 32) {
      const int64_t e = e0 + lane;
      int64_t f0 = 0, f1 = 0;
      uint64_t vb = 0;
      if (e < ptr[r + 1]) {
        const int j = idx[e];
        f0 = fptr[j];
        f1 = fptr[j + 1];
        vb = dtype == 0 ? (uint64_t)static_cast<const uint32_t*>(val)[e]
                        : (uint64_t)__double_as_longlong(static_cast<const double*>(val)[e]);
      }
      // this lane's records start after the lower lanes' (column order)
      int64_t c = f1 - f0, incl = c;
      for (int d = 1; d < 32; d <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += y;
      }
      const int64_t at = o + incl - c;
      for (int64_t q = f0; q < f1; ++q) {
        keys[at + (q - f0)] = ((uint64_t)r << rbits) | (uint64_t)(uint32_t)freg[q];
        vals[at + (q - f0)] = vb;
      }
      o += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
}

__global__ void agg_heads_kernel(int64_t E, const uint64_t* __restrict__ keys, int64_t* __restrict__ head) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x)
    head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

// at each run head: the run's sum into its output slot, its row counted
__global__ void agg_reduce_kernel(int64_t E, const uint64_t* __restrict__ keys, const uint64_t* __restrict__ vals,
                                  const int64_t* __restrict__ pos, int dtype, int rbits, int32_t* __restrict__ out_idx,
                                  void* __restrict__ out_val, int64_t cap, unsigned long long* __restrict__ rowcnt,
                                  int* __restrict__ status) {
  const uint64_t rmask = (1ull << rbits) - 1ull;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < E; i += (int64_t)gridDim.x * blockDim.x) {
    if (i > 0 && keys[i] == keys[i - 1]) continue;
    const int64_t p = pos[i] - 1;
    const uint64_t key = keys[i];
    int64_t j = i;
    if (dtype == 0) {
      uint64_t s = 0;
      for (; j < E && keys[j] == key; ++j) s += vals[j];
      if (s > 0xffffffffull) report_error(status, nullptr, SG_ERR_CONVERT, (unsigned long long)i);
      if (p < cap) static_cast<uint32_t*>(out_val)[p] = (uint32_t)s;
    } else {
      double s = 0.0;
      for (; j < E && keys[j] == key; ++j) s += __longlong_as_double((long long)vals[j]);
      if (p < cap) static_cast<double*>(out_val)[p] = s;
    }
    if (p < cap) out_idx[p] = (int32_t)(key & rmask);
    atomicAdd(rowcnt + (key >> rbits) + 1, 1ull);
  }
}

struct AggLayout {
  uint64_t *keys, *vals, *keys_alt, *vals_alt;
  int64_t* pos;
  void* radix;
  void* scan;
  int64_t bytes;
};

AggLayout agg_layout(char* base, int64_t E, int64_t n) {
  AggLayout L{};
  int64_t o = 0;
  auto take = [&](int64_t b) { const int64_t r = o; o += (b + 255) / 256 * 256; return r; };
  const int64_t E1 = E > 0 ? E : 1;
  const int64_t ok = take(8 * E1), ov = take(8 * E1), oka = take(8 * E1), ova = take(8 * E1), op = take(8 * E1),
                orad = take(radix_scratch_bytes(E1)), osc = take(scan_scratch_bytes((E1 > n + 1 ? E1 : n + 1)));
  if (base) {
    L.keys = (uint64_t*)(base + ok);
    L.vals = (uint64_t*)(base + ov);
    L.keys_alt = (uint64_t*)(base + oka);
    L.vals_alt = (uint64_t*)(base + ova);
    L.pos = (int64_t*)(base + op);
    L.radix = base + orad;
    L.scan = base + osc;
  }
  L.bytes = o;
  return L;
}

int bits_for(int64_t v) {  // bits to hold 0..v-1
  int b = 1;
  while (b < 63 && (int64_t(1) << b) < v) ++b;
  return b;
}

int sm_count_a() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_csr_aggregate_count(int64_t n, const int64_t* indptr, const int32_t* indices, const int64_t* fptr,
                                      int64_t* eoff, void* scan_scratch, void* stream) {
  if (n < 0 || (n > 0 && (!indptr || !indices || !fptr || !eoff || !scan_scratch))) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (n == 0) return cudaMemsetAsync(eoff, 0, sizeof(int64_t), s) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
  agg_count_kernel<<<grid_for(n * 32, 256, 8 * sm_count_a()), 256, 0, s>>>(n, indptr, indices, fptr, eoff);
  SG_CHECK_LAUNCH();
  return inclusive_scan_i64(eoff, n + 1, scan_scratch, s) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

extern "C" int64_t sg_csr_aggregate_scratch_bytes(int64_t n, int64_t n_records) {
  if (n < 0 || n_records < 0) return -1;
  return agg_layout(nullptr, n_records, n).bytes;
}

extern "C" int sg_csr_aggregate_run(int dtype, int64_t n, const int64_t* indptr, const int32_t* indices,
                                    const void* values, const int64_t* fptr, const int32_t* fregion,
                                    int64_t n_regions, const int64_t* eoff, int64_t n_records, void* scratch,
                                    int64_t scratch_bytes, int64_t* out_indptr, int32_t* out_idx, void* out_val,
                                    int64_t cap, int64_t* out_nnz, int* status, void* stream) {
  if ((dtype != 0 && dtype != 1) || n < 0 || n_regions < 0 || n_regions > (int64_t(1) << 31) || n_records < 0 ||
      !out_indptr || !out_nnz || !status || (n > 0 && (!indptr || !indices || !values || !fptr || !eoff)))
    return SG_ERR_ARG;
  if (((uintptr_t)scratch & 255u) != 0) return SG_ERR_ARG;
  AggLayout L = agg_layout((char*)scratch, n_records, n);
  if (scratch_bytes < L.bytes) return SG_ERR_CAP;
  const int rbits = bits_for(n_regions > 1 ? n_regions : 2);
  const int nbits = bits_for(n > 1 ? n : 2);
  if (rbits + nbits > 64) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(out_indptr, 0, sizeof(int64_t) * (n + 1), s) != cudaSuccess) return SG_ERR_CUDA;
  const int g = grid_for(n * 32, 256, 8 * sm_count_a());
  int64_t nnz = 0;
  if (n_records > 0) {
    agg_expand_kernel<<<g, 256, 0, s>>>(n, indptr, indices, values, dtype, fptr, fregion, eoff, rbits, L.keys,
                                        L.vals);
    SG_CHECK_LAUNCH();
    bool alt = false;
    if (radix_sort_u64(n_records, L.keys, L.vals, L.keys_alt, L.vals_alt, 0, rbits + nbits, L.radix, s, &alt) !=
        cudaSuccess)
      return SG_ERR_CUDA;
    const uint64_t* K = alt ? L.keys_alt : L.keys;
    const uint64_t* Vv = alt ? L.vals_alt : L.vals;
    const int ge = grid_for(n_records, 256, 16 * sm_count_a());
    agg_heads_kernel<<<ge, 256, 0, s>>>(n_records, K, L.pos);
    SG_CHECK_LAUNCH();
    if (inclusive_scan_i64(L.pos, n_records, L.scan, s) != cudaSuccess) return SG_ERR_CUDA;
    if (cudaMemcpyAsync(&nnz, L.pos + n_records - 1, sizeof(int64_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return SG_ERR_CUDA;
    if (nnz > cap) {
      *out_nnz = nnz;
      return SG_ERR_CAP;
    }
    agg_reduce_kernel<<<ge, 256, 0, s>>>(n_records, K, Vv, L.pos, dtype, rbits, out_idx, out_val, cap,
                                         reinterpret_cast<unsigned long long*>(out_indptr), status);
    SG_CHECK_LAUNCH();
  }
  if (n > 0 && inclusive_scan_i64(out_indptr, n + 1, L.scan, s) != cudaSuccess) return SG_ERR_CUDA;
  *out_nnz = nnz;
  return SG_OK;
}
