// Stage-tiled CSR SpMM: the dense operand is staged through shared memory.
//
//   out[r,:] = scale[r] * sum_{e in row r} val_e * in[col_e,:]  (- dshift[r] * y[r,:])
//
// Same contract as sg_spmm_masked (spectral.cu), different schedule.  The
// gather-per-nonzero kernel there reads every operand row through L1/L2; at
// block 8 FP32 each nonzero is one 32-byte row of its own 128-byte line, and
// random gathers of that shape run at about one line per SM clock (the L1
// tag rate), ~9 TB/s on GB300.  Shared memory serves ~4 such rows per
// clock before bank conflicts (~1.9 after them).
//
// Here each CTA (1024 threads, one per SM and wave) owns a contiguous range
// of rows and walks the operand in column stages of `stage_cols` rows.  A
// stage is copied global -> shared by bulk asynchronous copies (cp.async.bulk
// completing on an mbarrier), double-buffered so the next stage streams in
// while this one is consumed.  With the operand stage comes the stage's
// segment table: for every row of the range, the [start, end) of its
// nonzeros whose column falls in the stage (rows are sorted, so each row's
// part in a stage is contiguous).  The table is built once per operator
// (sg_staged_table); with it every index load of a row's segment has a known
// address, so all of them are in flight at once and only the gathers, from
// shared memory, depend on them.
//
// Work split: groups of SGL lanes own rows (row rr of the range goes to group
// rr mod groups, for every stage); inside a group LPN lanes cover the B
// values of one gathered row as 16-byte vectors, so a group step consumes
// SGL/LPN nonzeros (times the unroll U).  Partial sums of a row are combined
// by a fixed xor-shuffle tree inside the group, then added to the row's
// accumulator in stage order: shared memory when the range's accumulators fit
// (<= 64 KB), else the output row itself (L2-resident read-modify-write,
// owned by one group, so no atomics).  Results are deterministic; the
// summation order differs from the gather kernel's (rounding-level only).
//
// Rows with row_mask[r] == 0 are skipped and not written.  Column indices
// outside [0, cols) are left out of the table, so never gathered.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kStagedThreads = 1024;
constexpr int kStagedVariants = 4;
constexpr int64_t kMaxRowsPerCta = 4096;
constexpr int kAccSmemBytes = 64 * 1024;
constexpr int kHeader = 128;               // two mbarriers, padded

// Segment table of tile (cta j, stage k): starts[rpc4] then ends[rpc4] (u32,
// relative to ptr[first row of the range]) at offset (j * S + k) * 2 * rpc4.
struct StagedPlan {
  int64_t rows_per_cta, rpc4, grid, stage_cols, stages;
  int acc_smem;
  size_t smem;
};

int max_optin_smem() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return v;
}

int sm_count_staged() {
  int dev = 0, v = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
  return v > 0 ? v : 1;
}

// Rows split evenly over whole waves of CTAs (at most kMaxRowsPerCta each);
// the shared memory left after the two segment tables (and the accumulators
// when they fit) holds two operand stages.
bool plan_staged(int64_t rows, int64_t cols, int rowb, StagedPlan& pl) {
  if (rows < 1 || cols < 1) return false;
  const int64_t sms = sm_count_staged();
  const int64_t waves = (rows + sms * kMaxRowsPerCta - 1) / (sms * kMaxRowsPerCta);
  int64_t rpc = (rows + sms * waves - 1) / (sms * waves);
  if (rpc < 1) rpc = 1;
  pl.rows_per_cta = rpc;
  pl.rpc4 = (rpc + 3) / 4 * 4;
  pl.grid = (rows + rpc - 1) / rpc;
  pl.acc_smem = rpc * rowb <= kAccSmemBytes ? 1 : 0;
  const size_t seg = (size_t)pl.rpc4 * 8;
  const size_t fixed = kHeader + 2 * seg + (pl.acc_smem ? (size_t)rpc * rowb : 0);
  const int64_t avail = (int64_t)max_optin_smem() - (int64_t)fixed;
  if (avail <= 0) return false;
  int64_t st = avail / (2 * rowb);
  if (st >= cols) st = cols;  // the whole operand is one stage
  if (st < 64 && st < cols) return false;
  pl.stage_cols = st;
  pl.stages = (cols + st - 1) / st;
  pl.smem = fixed + 2 * (size_t)st * rowb;
  return true;
}

// Table build, one warp per row: a nonzero whose stage differs from its left
// neighbour's starts the row's segment of that stage, one whose stage differs
// from its right neighbour's ends it.  The table is zeroed first, so stages
// a row has no nonzero in have start = end = 0.
__global__ void staged_table_kernel(int64_t rows, int64_t cols, const int64_t* __restrict__ ptr,
                                    const int32_t* __restrict__ idx, int64_t rpc, int64_t rpc4, int64_t S,
                                    int64_t stage_cols, uint32_t* __restrict__ table) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < rows; r += nw) {
    const int64_t j = r / rpc, rr = r - j * rpc;
    const int64_t base = ptr[j * rpc];
    const int64_t s = ptr[r], e = ptr[r + 1];
    auto stage_of = [&](int64_t q) -> int64_t {
      const int64_t c = idx[q];
      return (c < 0 || c >= cols) ? -1 : c / stage_cols;
    };
    for (int64_t q0 = s; q0 < e; q0 += 32) {
      const int64_t q = q0 + lane;
      if (q >= e) continue;
      const int64_t k = stage_of(q);
      if (k < 0) continue;
      const int64_t kp = q == s ? -2 : stage_of(q - 1);
      const int64_t kn = q + 1 == e ? -2 : stage_of(q + 1);
      uint32_t* tile = table + (size_t)(j * S + k) * 2 * rpc4;
      if (k != kp) tile[rr] = (uint32_t)(q - base);
      if (k != kn) tile[rpc4 + rr] = (uint32_t)(q + 1 - base);
    }
  }
}

// Failure injection for tests (set only by sg_test_staged_fault): the stage
// whose copies thread 0 does not issue, so its barrier never completes and
// nothing is in flight for it, and the limit of every stage wait.  -1 and
// kWaitNs in normal operation.
__device__ int g_staged_skip_stage = -1;
__device__ unsigned long long g_staged_wait_ns = kWaitNs;

template <typename T, int B, bool VALUED, int SGL, int U>
__global__ void __launch_bounds__(kStagedThreads, 1)
spmm_staged_kernel(int64_t rows, int64_t cols, int64_t rows_per_cta, int64_t rpc4, int64_t stage_cols,
                   int acc_smem, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                   const float* __restrict__ val, const uint32_t* __restrict__ table, const T* __restrict__ in,
                   T* __restrict__ out, const T* __restrict__ scale, const T* __restrict__ dshift,
                   const T* __restrict__ y, const unsigned char* __restrict__ row_mask, int* __restrict__ status) {
  using VT = typename V16<T>::type;
  constexpr int VW = V16<T>::n;
  constexpr int LPN = B / VW;     // lanes per gathered row
  constexpr int PPG = SGL / LPN;  // nonzeros per group step and unroll slot
  constexpr int ROWB = B * (int)sizeof(T);
  static_assert(B % VW == 0 && LPN <= SGL && SGL <= 32 && (SGL & (SGL - 1)) == 0, "bad group shape");

  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
  const int64_t r0 = (int64_t)blockIdx.x * rows_per_cta;
  if (r0 >= rows) return;  // whole CTA, before any barrier is touched
  const int nr = (int)min(rows_per_cta, rows - r0);
  const int64_t S = (cols + stage_cols - 1) / stage_cols;
  const size_t stage_bytes = (size_t)stage_cols * ROWB;
  const size_t seg_bytes = (size_t)rpc4 * 8;
  unsigned char* ops = smem + kHeader;                                     // 2 operand stages
  uint32_t* segs = reinterpret_cast<uint32_t*>(ops + 2 * stage_bytes);     // 2 segment tables
  VT* sacc = reinterpret_cast<VT*>(reinterpret_cast<unsigned char*>(segs) + 2 * seg_bytes);
  const int64_t base = ptr[r0];
  const int32_t* ridx = idx + base;
  const float* rval = VALUED ? val + base : nullptr;

  const int64_t skip_stage = g_staged_skip_stage;
  const uint64_t wait_ns = g_staged_wait_ns;
  auto issue = [&](int64_t k) {
    if (k == skip_stage) return;  // test hook: this stage's barrier never completes
    const int64_t lo = k * stage_cols;
    const int64_t cnt = min(stage_cols, cols - lo);
    uint64_t* b = &bar[k & 1];
    const uint32_t opb = (uint32_t)(cnt * ROWB);
    mbar_expect_tx(b, opb + (uint32_t)seg_bytes);
    bulk_copy(ops + (size_t)(k & 1) * stage_bytes, in + lo * B, opb, b);
    bulk_copy(reinterpret_cast<unsigned char*>(segs) + (size_t)(k & 1) * seg_bytes,
              table + (size_t)(blockIdx.x * S + k) * 2 * rpc4, (uint32_t)seg_bytes, b);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_barrier_init();
    fence_proxy_async();
    issue(0);
    if (S > 1) issue(1);
  }
  if (acc_smem)
    for (int t = threadIdx.x; t < nr * LPN; t += blockDim.x) sacc[t] = V16<T>::zero();
  __syncthreads();

  const int lane = threadIdx.x & 31;
  const int gl = lane & (SGL - 1);
  const int pair = gl / LPN, sub = gl % LPN;
  const unsigned gmask = SGL == 32 ? 0xffffffffu : (((1u << SGL) - 1u) << (lane & ~(SGL - 1)));
  const int grp = threadIdx.x / SGL;
  constexpr int kGroups = kStagedThreads / SGL;

  for (int64_t k = 0; k < S; ++k) {
    const bool ok = mbar_wait(&bar[k & 1], (uint32_t)((k >> 1) & 1), wait_ns);
    if (!__syncthreads_and(ok)) {
      if (threadIdx.x == 0) {
        report_error(status, nullptr, SG_ERR_TIMEOUT, 0);
        // the other buffer's copies, if in flight: wait for them (bounded)
        if (k + 1 < S && k + 1 != skip_stage) mbar_wait(&bar[(k + 1) & 1], (uint32_t)(((k + 1) >> 1) & 1), wait_ns);
      }
      return;
    }
    const VT* sv = reinterpret_cast<const VT*>(ops + (size_t)(k & 1) * stage_bytes);
    const uint32_t* st = segs + (size_t)(k & 1) * 2 * rpc4;
    const int64_t lo = k * stage_cols;
    const uint32_t width = (uint32_t)min(stage_cols, cols - lo);
    const bool last = k == S - 1;
    for (int rr = grp; rr < nr; rr += kGroups) {
      const int64_t r = r0 + rr;
      if (row_mask && !row_mask[r]) continue;  // group-uniform
      const uint32_t a0 = st[rr], a1 = st[rpc4 + rr];
      VT prev = V16<T>::zero();
      if (!acc_smem && k > 0 && pair == 0) prev = __ldcg(reinterpret_cast<const VT*>(out + r * B) + sub);
      VT acc = V16<T>::zero();
      for (uint32_t t0 = a0; t0 < a1; t0 += PPG * U) {
        uint32_t loc[U];
        float v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          const uint32_t q = t0 + u * PPG + pair;
          loc[u] = q < a1 ? (uint32_t)((int64_t)__ldg(ridx + q) - lo) : 0xffffffffu;
          v[u] = (VALUED && q < a1) ? __ldg(rval + q) : 1.0f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
          if (loc[u] < width) {
            const VT g = sv[(size_t)loc[u] * LPN + sub];
            if (VALUED) V16<T>::fma(acc, (T)v[u], g);
            else V16<T>::add(acc, g);
          }
        }
      }
#pragma unroll
      for (int o = LPN; o < SGL; o <<= 1) {
        if constexpr (sizeof(T) == 4) {
          acc.x += __shfl_xor_sync(gmask, acc.x, o);
          acc.y += __shfl_xor_sync(gmask, acc.y, o);
          acc.z += __shfl_xor_sync(gmask, acc.z, o);
          acc.w += __shfl_xor_sync(gmask, acc.w, o);
        } else {
          acc.x += __shfl_xor_sync(gmask, acc.x, o);
          acc.y += __shfl_xor_sync(gmask, acc.y, o);
        }
      }
      if (pair == 0) {
        VT a = acc_smem ? sacc[(size_t)rr * LPN + sub] : prev;
        V16<T>::add(a, acc);
        if (last) {
          const T sc = scale[r];
          const T* av = reinterpret_cast<const T*>(&a);
          VT o;
          T* ov = reinterpret_cast<T*>(&o);
          if (dshift) {
            const T d = dshift[r];
            const VT yv = *(reinterpret_cast<const VT*>(y + r * B) + sub);
            const T* yp = reinterpret_cast<const T*>(&yv);
#pragma unroll
            for (int q = 0; q < VW; ++q) ov[q] = sc * av[q] - d * yp[q];
          } else {
#pragma unroll
            for (int q = 0; q < VW; ++q) ov[q] = sc * av[q];
          }
          *(reinterpret_cast<VT*>(out + r * B) + sub) = o;
        } else if (acc_smem) {
          sacc[(size_t)rr * LPN + sub] = a;
        } else {
          __stcg(reinterpret_cast<VT*>(out + r * B) + sub, a);
        }
      }
    }
    __syncthreads();  // every group is done with this buffer
    if (threadIdx.x == 0 && k + 2 < S) {
      fence_proxy_async();
      issue(k + 2);
    }
  }
}

template <typename T, int B, bool VALUED, int SGL, int U>
int launch_staged_v(int64_t rows, int64_t cols, const int64_t* ptr, const int32_t* idx, const float* val,
                    const uint32_t* table, const T* in, T* out, const T* scale, const T* dshift, const T* y,
                    const unsigned char* mk, int* status, cudaStream_t s) {
  constexpr int ROWB = B * (int)sizeof(T);
  StagedPlan pl;
  if (!plan_staged(rows, cols, ROWB, pl)) return SG_ERR_ARG;
  auto kern = spmm_staged_kernel<T, B, VALUED, SGL, U>;
  // opt in to the device's full shared memory once per device (not per
  // launch, so no attribute call falls inside a stream capture)
  static unsigned configured = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 32) return SG_ERR_ARG;
  if (!(configured & (1u << dev))) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, max_optin_smem()) != cudaSuccess)
      return SG_ERR_CUDA;
    configured |= 1u << dev;
  }
  kern<<<(unsigned)pl.grid, kStagedThreads, pl.smem, s>>>(rows, cols, pl.rows_per_cta, pl.rpc4, pl.stage_cols,
                                                          pl.acc_smem, ptr, idx, val, table, in, out, scale,
                                                          dshift, y, mk, status);
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

// variant -> (lanes per row group, unroll); the group never gets narrower
// than one gathered row (LPN lanes).
template <typename T, int B, bool VALUED>
int launch_staged_t(int variant, int64_t rows, int64_t cols, const int64_t* ptr, const int32_t* idx,
                    const float* val, const uint32_t* table, const T* in, T* out, const T* scale, const T* dshift,
                    const T* y, const unsigned char* mk, int* status, cudaStream_t s) {
  constexpr int LPN = B / V16<T>::n;
  constexpr int G8 = LPN > 8 ? LPN : 8;
  constexpr int G16 = LPN > 16 ? LPN : 16;
  switch (variant) {
    case 0: return launch_staged_v<T, B, VALUED, G8, 4>(rows, cols, ptr, idx, val, table, in, out, scale, dshift, y, mk, status, s);
    case 1: return launch_staged_v<T, B, VALUED, G8, 2>(rows, cols, ptr, idx, val, table, in, out, scale, dshift, y, mk, status, s);
    case 2: return launch_staged_v<T, B, VALUED, G16, 2>(rows, cols, ptr, idx, val, table, in, out, scale, dshift, y, mk, status, s);
    case 3: return launch_staged_v<T, B, VALUED, 32, 1>(rows, cols, ptr, idx, val, table, in, out, scale, dshift, y, mk, status, s);
    default: return SG_ERR_ARG;
  }
}

template <typename T>
int launch_staged(int variant, int B, int64_t rows, int64_t cols, const int64_t* ptr, const int32_t* idx,
                  const float* val, const uint32_t* table, const T* in, T* out, const T* scale, const T* dshift,
                  const T* y, const unsigned char* mk, int* status, cudaStream_t s) {
#define SG_STAGED_B(BB)                                                                                       \
  case BB:                                                                                                    \
    return val ? launch_staged_t<T, BB, true>(variant, rows, cols, ptr, idx, val, table, in, out, scale,      \
                                              dshift, y, mk, status, s)                                       \
               : launch_staged_t<T, BB, false>(variant, rows, cols, ptr, idx, val, table, in, out, scale,     \
                                               dshift, y, mk, status, s);
  switch (B) {
    SG_STAGED_B(4)
    SG_STAGED_B(8)
    SG_STAGED_B(16)
    SG_STAGED_B(32)
    default: return SG_ERR_ARG;
  }
#undef SG_STAGED_B
}

int row_bytes(int dtype, int block) {
  if ((dtype != 0 && dtype != 1) || (block != 4 && block != 8 && block != 16 && block != 32)) return 0;
  return block * (dtype == 0 ? 4 : 8);
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_spmm_staged_variants(void) { return kStagedVariants; }

extern "C" int64_t sg_staged_table_bytes(int dtype, int block, int64_t rows, int64_t cols) {
  const int rb = row_bytes(dtype, block);
  StagedPlan pl;
  if (!rb || !plan_staged(rows, cols, rb, pl)) return 0;
  return pl.grid * pl.stages * 2 * pl.rpc4 * 4;
}

extern "C" int sg_staged_table(int dtype, int block, int64_t rows, int64_t cols, const int64_t* ptr,
                               const int32_t* idx, void* table, int64_t table_bytes, void* stream) {
  const int rb = row_bytes(dtype, block);
  StagedPlan pl;
  if (!rb || !ptr || !idx || !table || !plan_staged(rows, cols, rb, pl)) return SG_ERR_ARG;
  const int64_t need = pl.grid * pl.stages * 2 * pl.rpc4 * 4;
  if (table_bytes < need) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  if (cudaMemsetAsync(table, 0, (size_t)need, s) != cudaSuccess) return SG_ERR_CUDA;
  staged_table_kernel<<<grid_for(rows * 32, 256, 32 * sm_count_staged()), 256, 0, s>>>(
      rows, cols, ptr, idx, pl.rows_per_cta, pl.rpc4, pl.stages, pl.stage_cols, static_cast<uint32_t*>(table));
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_spmm_staged(int dtype, int block, int64_t rows, int64_t cols, const int64_t* ptr,
                              const int32_t* idx, const float* val, const void* table, const void* in, void* out,
                              const void* scale, const void* dshift, const void* y, int variant,
                              const unsigned char* row_mask, int* status, void* stream) {
  if (rows < 0 || cols < 1 || !ptr || !idx || !table || !in || !out || !scale || (dshift && !y) || !status ||
      variant < 0 || variant >= kStagedVariants)
    return SG_ERR_ARG;
  if ((reinterpret_cast<uintptr_t>(in) & 15) || (reinterpret_cast<uintptr_t>(out) & 15) ||
      (reinterpret_cast<uintptr_t>(table) & 15) || (y && (reinterpret_cast<uintptr_t>(y) & 15)))
    return SG_ERR_ARG;
  if (rows == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  const uint32_t* tb = static_cast<const uint32_t*>(table);
  if (dtype == 0)
    return launch_staged<float>(variant, block, rows, cols, ptr, idx, val, tb, (const float*)in, (float*)out,
                                (const float*)scale, (const float*)dshift, (const float*)y, row_mask, status, s);
  if (dtype == 1)
    return launch_staged<double>(variant, block, rows, cols, ptr, idx, val, tb, (const double*)in, (double*)out,
                                 (const double*)scale, (const double*)dshift, (const double*)y, row_mask, status,
                                 s);
  return SG_ERR_ARG;
}

// Test hook: make the stage-tiled SpMM skip the copies of one stage (so its
// bounded wait runs out with nothing in flight) and shorten the wait limit;
// skip_stage < 0 and wait_ns <= 0 restore normal operation.  Synchronous.
extern "C" int sg_test_staged_fault(int skip_stage, int64_t wait_ns) {
  const int v = skip_stage < 0 ? -1 : skip_stage;
  const unsigned long long ns = wait_ns > 0 ? (unsigned long long)wait_ns : kWaitNs;
  if (cudaMemcpyToSymbol(g_staged_skip_stage, &v, sizeof(v)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_staged_wait_ns, &ns, sizeof(ns)) != cudaSuccess)
    return SG_ERR_CUDA;
  return SG_OK;
}
