// Cell-by-region counts (peak matrix): fragments -> CSR of region hit
// counts, the arithmetic of RegionCounter::insert_fragment
// (snapatac2-core/src/feature_count/counter.rs:117-146) over the fragments
// that pair_to_fragments / single_to_fragments rebuild
// (snapatac2-core/src/feature_count/data_iter.rs:27-117), driven by
// create_peak_matrix (snapatac2-core/src/feature_count/matrix.rs:95-170).
//
// Regions are given per chromosome, sorted by start, with the running
// maximum of their ends: the regions that overlap [qs, qe) are found by one
// binary search (last start < qe) and a backward scan that stops when the
// running maximum end falls to qs or below.
//
// Same three-phase layout as the tile matrix (one CTA per cell): plan counts
// the region hits ("keys") per cell; run regenerates them into shared memory
// (global scratch for long rows), sorts them (CTA radix sort over the bits
// the row spans) and run-length encodes them into (region, count) pairs;
// sg_tile_emit compacts the pairs into the CSR arrays (same scratch layout).
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kPlanBlock = 256;
constexpr int kRunBlock = 512;
constexpr int kSmemKeys = 24576;

struct RegionSet {
  const uint64_t* __restrict__ chrom_end;  // cumulative chromosome lengths
  const uint8_t* __restrict__ excl;
  int n_chrom;
  const int64_t* __restrict__ rptr;   // regions of chromosome c: [rptr[c], rptr[c + 1])
  const uint64_t* __restrict__ rs;    // start (0-based, chromosome coordinates)
  const uint64_t* __restrict__ re;    // end (exclusive)
  const uint64_t* __restrict__ rmax;  // running max of re within the chromosome
  const uint32_t* __restrict__ rid;   // feature index
};

struct RFilter {
  int strategy;
  int64_t min_len, max_len;
};

// regions overlapping [qs, qe) of chromosome c; `skip` > 0 drops those that
// also contain the point skip_at (the paired-insertion union)
template <class F>
__device__ __forceinline__ void visit(const RegionSet& R, int c, uint64_t qs, uint64_t qe, bool skip,
                                      uint64_t skip_at, F&& f) {
  const int64_t lo = R.rptr[c], hi = R.rptr[c + 1];
  int64_t a = lo, b = hi;  // first region with start >= qe
  while (a < b) {
    const int64_t m = (a + b) >> 1;
    if (__ldg(R.rs + m) < qe) a = m + 1;
    else b = m;
  }
  for (int64_t j = a - 1; j >= lo; --j) {
    if (__ldg(R.rmax + j) <= qs) break;
    const uint64_t e = __ldg(R.re + j);
    if (e > qs) {
      if (skip && __ldg(R.rs + j) <= skip_at && e > skip_at) continue;
      f(__ldg(R.rid + j));
    }
  }
}

// Hits of one fragment: returns their number (calling f for each), or -1
// when the position lies outside the genome.
template <class F>
__device__ __forceinline__ int fragment_hits(const RegionSet& R, const RFilter& flt, uint64_t pos, uint32_t len,
                                             F&& f) {
  int a = 0, b = R.n_chrom;  // first chromosome with end > pos
  while (a < b) {
    const int m = (a + b) >> 1;
    if (__ldg(R.chrom_end + m) <= pos) a = m + 1;
    else b = m;
  }
  if (a >= R.n_chrom) return -1;
  if (__ldg(R.excl + a)) return 0;
  const uint64_t s = pos - (a ? __ldg(R.chrom_end + a - 1) : 0ull);
  int n = 0;
  auto g = [&](uint32_t k) {
    ++n;
    f(k);
  };
  if (flt.strategy == SG_COUNT_SINGLE) {
    visit(R, a, s, s + 1, false, 0, g);
    return n;
  }
  const uint64_t size = len;
  if (flt.min_len >= 0 && size < (uint64_t)flt.min_len) return 0;
  if (flt.max_len >= 0 && size > (uint64_t)flt.max_len) return 0;
  const uint64_t e = s + size, e1 = e - 1ull;  // wraps like the reference's u64
  switch (flt.strategy) {
    case SG_COUNT_FRAGMENT: visit(R, a, s, e, false, 0, g); break;
    case SG_COUNT_INSERTION:
      visit(R, a, s, s + 1, false, 0, g);
      visit(R, a, e1, e1 + 1, false, 0, g);
      break;
    default:  // paired-insertion: each region hit by either insertion once
      visit(R, a, s, s + 1, false, 0, g);
      visit(R, a, e1, e1 + 1, true, s, g);
      break;
  }
  return n;
}

__global__ void __launch_bounds__(kPlanBlock)
region_plan_kernel(const int64_t* __restrict__ cell_ptr, int64_t n_cells, int64_t n_frags,
                   const uint64_t* __restrict__ pos, const uint32_t* __restrict__ len, RegionSet R, RFilter flt,
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
    const int r = fragment_hits(R, flt, pos[k], len ? len[k] : 0u, [](uint32_t) {});
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
region_run_kernel(const int64_t* __restrict__ cell_ptr, int64_t n_cells, int64_t n_frags,
                  const uint64_t* __restrict__ pos, const uint32_t* __restrict__ len, RegionSet R, RFilter flt,
                  const int64_t* __restrict__ key_ptr, int64_t key_cap, uint32_t* __restrict__ gkeys,
                  uint32_t* __restrict__ gtmp, int32_t* __restrict__ pair_idx, uint32_t* __restrict__ pair_cnt,
                  int64_t* __restrict__ cell_nnz, int* status) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
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

  // 1. regenerate the cell's region hits (order is irrelevant before sorting)
  if (tid == 0) sm.fill = 0;
  __syncthreads();
  unsigned kmin = 0xffffffffu, kmax = 0u;
  for (int64_t k0 = fa; k0 < fb; k0 += kRunBlock) {
    const int64_t k = k0 + tid;
    int r = 0;
    if (k < fb) {
      r = fragment_hits(R, flt, pos[k], len ? len[k] : 0u, [](uint32_t) {});
      if (r < 0) r = 0;  // already reported by plan
    }
    int x = r;  // warp-aggregated slot reservation
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    int wbase = 0;
    if (lane == 31) wbase = atomicAdd(&sm.fill, x);
    wbase = __shfl_sync(0xffffffffu, wbase, 31);
    int o = wbase + x - r;
    if (r > 0 && o + r <= K) {
      fragment_hits(R, flt, pos[k], len ? len[k] : 0u, [&](uint32_t key) {
        A[o++] = key;
        kmin = min(kmin, key);
        kmax = max(kmax, key);
      });
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

  // 2. sort, 3. run-length encode: H[u] = start of the u-th distinct region
  uint32_t* S = cta_radix_sort<kRunBlock>(A, B, K, kmin, nbits, sm.sort);
  uint32_t* H = (S == A) ? B : A;
  int U = 0;
  for (int base = 0; base < K; base += kRunBlock) {
    const int i = base + tid;
    int head = 0;
    if (i < K) head = (i == 0) || (S[i] != S[i - 1]);
    int tot;
    const int p = block_exscan<kRunBlock>(head, sm.scan_ws, tot);
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

__global__ void zero_first_r(int64_t* p) { p[0] = 0; }

int check_region_args(int64_t n_cells, int n_chrom, int strategy, int64_t n_features) {
  if (n_cells < 0 || n_cells > 0x7fffffffLL || n_chrom <= 0) return SG_ERR_ARG;
  if (strategy < SG_COUNT_INSERTION || strategy > SG_COUNT_SINGLE) return SG_ERR_ARG;
  if (n_features < 0 || n_features > 0x7fffffffLL) return SG_ERR_ARG;
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_region_plan(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                              const uint32_t* frag_len, const uint64_t* chrom_end, const uint8_t* chrom_excl,
                              int n_chrom, const int64_t* region_ptr, const uint64_t* region_start,
                              const uint64_t* region_end, const uint64_t* region_maxend, const uint32_t* region_id,
                              int64_t n_features, int strategy, int64_t min_len, int64_t max_len, int64_t* key_ptr,
                              void* scan_scratch, int* status, unsigned long long* bad, void* stream) {
  const int e = check_region_args(n_cells, n_chrom, strategy, n_features);
  if (e) return e;
  if (strategy != SG_COUNT_SINGLE && !frag_len && n_frags > 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (n_cells == 0) {
    zero_first_r<<<1, 1, 0, s>>>(key_ptr);
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  RegionSet R{chrom_end, chrom_excl, n_chrom, region_ptr, region_start, region_end, region_maxend, region_id};
  RFilter f{strategy, min_len, max_len};
  region_plan_kernel<<<(unsigned)n_cells, kPlanBlock, 0, s>>>(cell_ptr, n_cells, n_frags, frag_pos,
                                                              strategy == SG_COUNT_SINGLE ? nullptr : frag_len, R,
                                                              f, key_ptr, status, bad);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(key_ptr + 1, n_cells, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}

extern "C" int sg_region_run(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                             const uint32_t* frag_len, const uint64_t* chrom_end, const uint8_t* chrom_excl,
                             int n_chrom, const int64_t* region_ptr, const uint64_t* region_start,
                             const uint64_t* region_end, const uint64_t* region_maxend, const uint32_t* region_id,
                             int64_t n_features, int strategy, int64_t min_len, int64_t max_len,
                             const int64_t* key_ptr, void* scratch, int64_t scratch_bytes, int64_t* out_indptr,
                             void* scan_scratch, int* status, unsigned long long* bad, void* stream) {
  (void)bad;
  const int e = check_region_args(n_cells, n_chrom, strategy, n_features);
  if (e) return e;
  if (strategy != SG_COUNT_SINGLE && !frag_len && n_frags > 0) return SG_ERR_ARG;
  if (((uintptr_t)scratch & 15u) != 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (n_cells == 0) {
    zero_first_r<<<1, 1, 0, s>>>(out_indptr);
    SG_CHECK_LAUNCH();
    return SG_OK;
  }
  // same sub-buffer split as sg_tile_run, so that sg_tile_emit reads the pairs
  const int64_t k4 = (scratch_bytes - 16) / (4 * (int64_t)sizeof(uint32_t));
  if (k4 < 0) return SG_ERR_CAP;
  uint32_t* base = reinterpret_cast<uint32_t*>(scratch);
  RegionSet R{chrom_end, chrom_excl, n_chrom, region_ptr, region_start, region_end, region_maxend, region_id};
  RFilter f{strategy, min_len, max_len};
  const size_t smem = sizeof(RunSmem) + 2 * (size_t)kSmemKeys * sizeof(uint32_t);
  if (cudaFuncSetAttribute(region_run_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  zero_first_r<<<1, 1, 0, s>>>(out_indptr);
  region_run_kernel<<<(unsigned)n_cells, kRunBlock, smem, s>>>(
      cell_ptr, n_cells, n_frags, frag_pos, strategy == SG_COUNT_SINGLE ? nullptr : frag_len, R, f, key_ptr, k4,
      base, base + k4, reinterpret_cast<int32_t*>(base + 2 * k4), base + 3 * k4, out_indptr, status);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(out_indptr + 1, n_cells, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}
