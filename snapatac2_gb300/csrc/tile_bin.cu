// Tile binning: fragments -> cell x tile count CSR, bit-exact with the
// reference's gen_mat_pair / gen_mat_single
// (snapatac2-core/src/feature_count/data_iter.rs:313-415).
//
// Design (one CTA per cell):
//   plan : every fragment is located on the genome (binary search of the
//          cumulative chromosome lengths, genome.rs:419-434), filtered
//          (excluded chromosome, size bounds) and checked (end past the
//          chromosome -> SG_ERR_RANGE, the reference's panic in
//          get_position_rev, genome.rs:397-399); the number of tile hits is
//          summed per cell and prefix-summed into key_ptr.
//   run  : the CTA regenerates the cell's tile hits ("keys") into shared
//          memory (or into global scratch for cells above kSmemKeys), sorts
//          them with a stable LSD radix sort over the bits spanned by the
//          cell, and run-length encodes them into (tile, count) pairs.  The
//          per-cell unique counts are prefix-summed into out_indptr.
//   emit : pairs are compacted from the key_ptr layout into the CSR arrays.
// The BTreeMap of the reference yields tiles in increasing order with their
// hit counts; sorting + run-length encoding yields exactly the same rows.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kPlanBlock = 256;
constexpr int kRunBlock = 512;
constexpr int kSmemKeys = 24576;  // keys per cell sorted in shared memory

struct Genome {
  const uint64_t* __restrict__ end;  // cumulative base lengths
  const uint64_t* __restrict__ bin_off;
  const uint8_t* __restrict__ excl;
  int n;
  uint32_t bin;
};

struct Filter {
  int strategy;
  int64_t min_len, max_len;
};

// Fragment -> [lo, hi] tile range plus the number of keys it emits.
// Returns 0 (skipped), the key count, or -1 on a range error.
__device__ __forceinline__ int frag_keys(const Genome& g, const Filter& f, uint64_t pos,
                                         uint32_t len, uint32_t& lo, uint32_t& hi) {
  int a = 0, b = g.n;  // first chromosome with end > pos
  while (a < b) {
    int m = (a + b) >> 1;
    if (__ldg(g.end + m) <= pos) a = m + 1; else b = m;
  }
  if (a >= g.n) return -1;
  const uint64_t cstart = a ? __ldg(g.end + a - 1) : 0ull;
  const uint64_t start = pos - cstart;
  if (__ldg(g.excl + a)) return 0;
  const uint64_t off = __ldg(g.bin_off + a);
  if (f.strategy == SG_COUNT_SINGLE) {
    lo = hi = (uint32_t)(off + (uint32_t)start / g.bin);
    return 1;
  }
  const uint64_t fs = len;
  const uint64_t end = start + fs - 1ull;  // wraps like the reference's u64
  if (f.min_len >= 0 && fs < (uint64_t)f.min_len) return 0;
  if (f.max_len >= 0 && fs > (uint64_t)f.max_len) return 0;
  const uint64_t csize = __ldg(g.end + a) - cstart;
  if (end >= csize) return -1;
  lo = (uint32_t)(off + (uint32_t)start / g.bin);
  hi = (uint32_t)(off + (uint32_t)end / g.bin);
  switch (f.strategy) {
    case SG_COUNT_INSERTION: return 2;
    case SG_COUNT_PIC: return hi != lo ? 2 : 1;
    default: return hi >= lo ? (int)(hi - lo + 1u) : 0;  // fragment
  }
}

__global__ void __launch_bounds__(kPlanBlock)
plan_kernel(const int64_t* __restrict__ cell_ptr, int64_t n_cells, int64_t n_frags,
            const uint64_t* __restrict__ pos, const uint32_t* __restrict__ len, Genome g, Filter f,
            int64_t* __restrict__ key_ptr, int* status, unsigned long long* bad) {
  __shared__ long long ws[kPlanBlock / 32];
  const int64_t c = blockIdx.x;
  if (c >= n_cells) return;
  int64_t a = cell_ptr[c], b = cell_ptr[c + 1];
  if (a < 0 || b < a || b > n_frags) {  // malformed row pointer: no access
    if (threadIdx.x == 0) report_error(status, nullptr, SG_ERR_ARG, 0);
    a = b = 0;
  }
  long long cnt = 0;
  for (int64_t k = a + threadIdx.x; k < b; k += kPlanBlock) {
    uint32_t lo, hi;
    int r = frag_keys(g, f, pos[k], len[k], lo, hi);
    if (r < 0) report_error(status, bad, SG_ERR_RANGE, (unsigned long long)k);
    else cnt += r;
  }
  cnt = block_sum_ll<kPlanBlock>(cnt, ws);
  if (threadIdx.x == 0) {
    key_ptr[c + 1] = cnt;
    if (c == 0) key_ptr[0] = 0;
  }
}

struct RunSmem {
  SortSmem<kRunBlock> sort;
  unsigned kmin_ws[kRunBlock / 32];
  int scan_ws[kRunBlock / 32 + 1];
  int fill;
};

__global__ void __launch_bounds__(kRunBlock)
run_kernel(const int64_t* __restrict__ cell_ptr, int64_t n_cells, int64_t n_frags,
           const uint64_t* __restrict__ pos, const uint32_t* __restrict__ len, Genome g, Filter f,
           const int64_t* __restrict__ key_ptr, int64_t key_cap, uint32_t* __restrict__ gkeys, uint32_t* __restrict__ gtmp, int32_t* __restrict__ pair_idx,
           uint32_t* __restrict__ pair_cnt, int64_t* __restrict__ cell_nnz, int* status) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RunSmem& sm = *reinterpret_cast<RunSmem*>(smem_raw);
  uint32_t* skeys = reinterpret_cast<uint32_t*>(smem_raw + sizeof(RunSmem));
  const int64_t c = blockIdx.x;
  if (c >= n_cells) return;
  const int tid = threadIdx.x, lane = tid & 31;
  const int64_t kbase = key_ptr[c];
  const int64_t K64 = key_ptr[c + 1] - kbase;
  const int64_t fa = cell_ptr[c], fb = cell_ptr[c + 1];
  if (K64 <= 0 || kbase < 0 || kbase + K64 > key_cap || K64 > 0x7fffffffLL || fa < 0 || fb < fa ||
      fb > n_frags) {
    if (tid == 0) {
      cell_nnz[c + 1] = 0;
      if (K64 != 0) report_error(status, nullptr, K64 < 0 ? SG_ERR_ARG : SG_ERR_CAP, 0);
    }
    return;
  }
  const int K = (int)K64;
  const bool in_smem = K <= kSmemKeys;
  uint32_t* A = in_smem ? skeys : gkeys + kbase;
  uint32_t* B = in_smem ? skeys + kSmemKeys : gtmp + kbase;

  // 1. regenerate the cell's tile hits; order is irrelevant before sorting
  if (tid == 0) sm.fill = 0;
  __syncthreads();
  unsigned kmin = 0xffffffffu, kmax = 0u;
  for (int64_t k0 = fa; k0 < fb; k0 += kRunBlock) {
    const int64_t k = k0 + tid;
    uint32_t lo = 0, hi = 0;
    int r = 0;
    if (k < fb) {
      r = frag_keys(g, f, pos[k], len[k], lo, hi);
      if (r < 0) r = 0;  // already reported by plan
    }
    // warp-aggregated slot reservation
    int x = r;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    int wbase = 0;
    if (lane == 31) wbase = atomicAdd(&sm.fill, x);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    int o = wbase + x - r;
    if (r > 0 && o + r <= K) {
      if (f.strategy == SG_COUNT_FRAGMENT) {
        for (uint32_t t = lo; t <= hi; ++t) A[o++] = t;
      } else if (f.strategy == SG_COUNT_INSERTION) {
        A[o] = lo;
        A[o + 1] = hi;
      } else {
        A[o] = lo;
        if (r == 2) A[o + 1] = hi;
      }
      // a zero-length fragment has hi = lo - 1 (end = start - 1)
      kmin = min(kmin, min(lo, hi));
      kmax = max(kmax, max(lo, hi));
    }
  }
  __syncthreads();
  if (sm.fill != K) {  // plan and run disagree: inputs changed in between
    if (tid == 0) {
      cell_nnz[c + 1] = 0;
      report_error(status, nullptr, SG_ERR_ARG, 0);
    }
    return;
  }
  kmin = block_min_u32<kRunBlock>(kmin, sm.kmin_ws);
  kmax = block_max_u32<kRunBlock>(kmax, sm.kmin_ws);
  const unsigned span = kmax - kmin;
  const int nbits = span ? 32 - __clz(span) : 0;

  // 2. sort
  uint32_t* S = cta_radix_sort<kRunBlock>(A, B, K, kmin, nbits, sm.sort);
  uint32_t* H = (S == A) ? B : A;  // free buffer: run starts

  // 3. run-length encode: H[u] = start of the u-th distinct tile
  int U = 0;
  for (int base = 0; base < K; base += kRunBlock) {
    const int i = base + tid;
    int head = 0;
    if (i < K) head = (i == 0) || (S[i] != S[i - 1]);
    int tot;
    int p = block_exscan<kRunBlock>(head, sm.scan_ws, tot);
    if (head) H[U + p] = (uint32_t)i;
    U += tot;
  }
  __syncthreads();
  int32_t* pi = pair_idx + kbase;
  uint32_t* pc = pair_cnt + kbase;
  for (int u = tid; u < U; u += kRunBlock) {
    const uint32_t s0 = H[u];
    const uint32_t s1 = (u + 1 < U) ? H[u + 1] : (uint32_t)K;
    pi[u] = (int32_t)S[s0];
    pc[u] = s1 - s0;
  }
  if (tid == 0) cell_nnz[c + 1] = U;
}

__global__ void emit_kernel(int64_t n_cells, const int64_t* __restrict__ key_ptr, int64_t key_cap,
                            const int32_t* __restrict__ pair_idx, const uint32_t* __restrict__ pair_cnt,
                            const int64_t* __restrict__ out_indptr, int32_t* __restrict__ out_idx,
                            uint32_t* __restrict__ out_cnt, int64_t cap, int* status) {
  const int64_t c = blockIdx.x;
  if (c >= n_cells) return;
  const int64_t src = key_ptr[c], dst = out_indptr[c], n = out_indptr[c + 1] - dst;
  if (dst < 0 || n < 0 || dst + n > cap || src < 0 || src + n > key_cap) {
    if (threadIdx.x == 0) report_error(status, nullptr, SG_ERR_CAP, 0);
    return;
  }
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
    out_idx[dst + i] = pair_idx[src + i];
    out_cnt[dst + i] = pair_cnt[src + i];
  }
}

__global__ void zero_first(int64_t* p) { p[0] = 0; }

}  // namespace
}  // namespace sg

using namespace sg;

static int check_common(int64_t n_cells, int n_chrom, uint32_t bin_size, int strategy) {
  if (n_cells < 0 || n_cells > 0x7fffffffLL || n_chrom <= 0 || bin_size == 0) return SG_ERR_ARG;
  if (strategy < SG_COUNT_INSERTION || strategy > SG_COUNT_SINGLE) return SG_ERR_ARG;
  return SG_OK;
}

extern "C" int64_t sg_scan_scratch_bytes(int64_t n) { return sg::scan_scratch_bytes(n); }

extern "C" int64_t sg_tile_scratch_bytes(int64_t total_keys) {
  if (total_keys < 0) return -1;
  // gkeys + gtmp (uint32) + pair_idx (int32) + pair_cnt (uint32) + cell_nnz scan
  // area is separate (out_indptr); 16-byte aligned sub-buffers.
  int64_t k = (total_keys + 3) / 4 * 4;
  return 4 * k * (int64_t)sizeof(uint32_t) + 16;
}

extern "C" int sg_tile_plan(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                            const uint32_t* frag_len, const uint64_t* chrom_end, const uint64_t* bin_off,
                            const uint8_t* chrom_excl, int n_chrom, uint32_t bin_size, int strategy,
                            int64_t min_len, int64_t max_len, int64_t* key_ptr, void* scan_scratch,
                            int* status, unsigned long long* bad, void* stream) {
  int e = check_common(n_cells, n_chrom, bin_size, strategy);
  if (e) return e;
  cudaStream_t s = as_stream(stream);
  if (n_cells == 0) {
    zero_first<<<1, 1, 0, s>>>(key_ptr);
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  Genome g{chrom_end, bin_off, chrom_excl, n_chrom, bin_size};
  Filter f{strategy, min_len, max_len};
  plan_kernel<<<(unsigned)n_cells, kPlanBlock, 0, s>>>(cell_ptr, n_cells, n_frags, frag_pos, frag_len,
                                                       g, f, key_ptr, status, bad);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(key_ptr + 1, n_cells, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}

extern "C" int sg_tile_run(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                           const uint32_t* frag_len, const uint64_t* chrom_end, const uint64_t* bin_off,
                           const uint8_t* chrom_excl, int n_chrom, uint32_t bin_size, int strategy,
                           int64_t min_len, int64_t max_len, const int64_t* key_ptr, void* scratch,
                           int64_t scratch_bytes, int64_t* out_indptr, void* scan_scratch, int* status,
                           unsigned long long* bad, void* stream) {
  (void)bad;
  int e = check_common(n_cells, n_chrom, bin_size, strategy);
  if (e) return e;
  if (((uintptr_t)scratch & 15u) != 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (n_cells == 0) {
    zero_first<<<1, 1, 0, s>>>(out_indptr);
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  // The caller sized scratch from key_ptr[n_cells]; the sub-buffer split uses
  // that same total, recovered from the byte count.
  const int64_t k4 = (scratch_bytes - 16) / (4 * (int64_t)sizeof(uint32_t));
  if (k4 < 0) return SG_ERR_CAP;
  uint32_t* base = reinterpret_cast<uint32_t*>(scratch);
  uint32_t* gkeys = base;
  uint32_t* gtmp = base + k4;
  int32_t* pidx = reinterpret_cast<int32_t*>(base + 2 * k4);
  uint32_t* pcnt = base + 3 * k4;
  Genome g{chrom_end, bin_off, chrom_excl, n_chrom, bin_size};
  Filter f{strategy, min_len, max_len};
  const size_t smem = sizeof(RunSmem) + 2 * (size_t)kSmemKeys * sizeof(uint32_t);
  // per function and device; cheap enough to set on every call
  if (cudaFuncSetAttribute(run_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  zero_first<<<1, 1, 0, s>>>(out_indptr);
  run_kernel<<<(unsigned)n_cells, kRunBlock, smem, s>>>(cell_ptr, n_cells, n_frags, frag_pos, frag_len,
                                                        g, f, key_ptr, k4, gkeys, gtmp, pidx, pcnt, out_indptr,
                                                        status);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(out_indptr + 1, n_cells, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}

extern "C" int sg_tile_emit(int64_t n_cells, const int64_t* key_ptr, const void* scratch,
                            int64_t scratch_bytes, const int64_t* out_indptr, int32_t* out_idx,
                            uint32_t* out_cnt, int64_t cap, int* status, void* stream) {
  if (n_cells < 0) return SG_ERR_ARG;
  if (n_cells == 0) return SG_OK;
  const int64_t k4 = (scratch_bytes - 16) / (4 * (int64_t)sizeof(uint32_t));
  if (k4 < 0) return SG_ERR_CAP;
  const uint32_t* base = reinterpret_cast<const uint32_t*>(scratch);
  emit_kernel<<<(unsigned)n_cells, 256, 0, as_stream(stream)>>>(
      n_cells, key_ptr, k4, reinterpret_cast<const int32_t*>(base + 2 * k4), base + 3 * k4, out_indptr,
      out_idx, out_cnt, cap, status);
  SG_CHECK_LAUNCH();
  return SG_OK;
}
