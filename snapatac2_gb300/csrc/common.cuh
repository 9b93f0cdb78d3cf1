// Shared device helpers for the snapgb300 kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "snapgb300.h"

#define SG_CHECK_LAUNCH()                                   \
  do {                                                      \
    cudaError_t e__ = cudaGetLastError();                   \
    if (e__ != cudaSuccess) return SG_ERR_CUDA;             \
  } while (0)

namespace sg {

constexpr int kWarp = 32;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// 16-byte vector of T (4 floats or 2 doubles): the unit of the SpMM gathers.
template <typename T> struct V16;
template <> struct V16<float> {
  using type = float4;
  static constexpr int n = 4;
  __device__ static float4 zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  __device__ static void add(float4& a, const float4& b) { a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w; }
  __device__ static void fma(float4& a, float s, const float4& b) {
    a.x = fmaf(s, b.x, a.x); a.y = fmaf(s, b.y, a.y); a.z = fmaf(s, b.z, a.z); a.w = fmaf(s, b.w, a.w);
  }
  __device__ static float4 shfl_xor(const float4& v, int o) {
    return make_float4(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o),
                       __shfl_xor_sync(0xffffffffu, v.z, o), __shfl_xor_sync(0xffffffffu, v.w, o));
  }
};
template <> struct V16<double> {
  using type = double2;
  static constexpr int n = 2;
  __device__ static double2 zero() { return make_double2(0.0, 0.0); }
  __device__ static void add(double2& a, const double2& b) { a.x += b.x; a.y += b.y; }
  __device__ static void fma(double2& a, double s, const double2& b) { a.x = ::fma(s, b.x, a.x); a.y = ::fma(s, b.y, a.y); }
  __device__ static double2 shfl_xor(const double2& v, int o) {
    return make_double2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o));
  }
};

// Column sums of a B-wide row block held as per-lane partials acc[0..B-1]:
// a transpose butterfly (lane pairs swap half of their sums at each step)
// leaves column c's total in acc[0] of the 32/B lanes whose high bits spell
// c, after B - 1 + 5 - log2(B) shuffles.  Fixed order: deterministic.
template <typename T, int B>
__device__ __forceinline__ void warp_colsum(T (&acc)[B], int lane) {
  // halve the columns a lane holds while doubling the lanes each sum covers
  int live = B;
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) {
    if (live > 1) {
      const int half = live / 2;
      const bool upper = (lane & o) != 0;
#pragma unroll
      for (int c = 0; c < B / 2; ++c) {
        if (c < half) {
          const T send = upper ? acc[c] : acc[c + half];
          const T recv = __shfl_xor_sync(0xffffffffu, send, o);
          acc[c] = (upper ? acc[c + half] : acc[c]) + recv;
        }
      }
      live = half;
    } else {
      acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], o);
    }
  }
}

// ---- mbarrier + bulk asynchronous copy (cp.async.bulk) helpers -----------
constexpr uint64_t kWaitNs = 2000000000ull;  // bounded mbarrier wait: 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses (and the
// block's, after a __syncthreads) before later async-proxy ones.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One bulk copy of `bytes` (multiple of 16, both addresses 16-byte aligned)
// global -> shared, completing its bytes on `bar` (armed by the caller).
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Plain arrival on `bar` (release: this thread's earlier shared-memory
// accesses are ordered before the phase completes).
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Arm `bar` for `bytes` of asynchronous copies (one arrival).
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// ---- tcgen05 (5th-generation tensor cores, TMEM accumulators) helpers ----
// Shared-memory matrix descriptor, no swizzle, K-major: the operand is an
// array of 8-row x 16-byte core matrices; `lbo` is the byte distance between
// core matrices along K, `sbo` between 8-row groups.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version of this generation
  return d;                // base offset 0, swizzle none
}

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator, bf16
// A and B, both K-major, M x N tile.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A[adesc] B[bdesc]^T, issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          bool accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate));
}

// Arrive once on `bar` when every tcgen05.mma this thread issued has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 columns of this warp's 32 TMEM lanes (one row per thread).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,"
      "%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Wait for the phase with this parity to complete; gives up (false) after
// limit_ns of wall time (kWaitNs by default), so a copy that never lands
// cannot hang the kernel.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitNs) {
  const uint64_t t0 = global_ns();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

// Record the first error: status word goes from 0 to `code`, and the lowest
// offending entry index is kept.
__device__ __forceinline__ void report_error(int* status, unsigned long long* bad, int code,
                                             unsigned long long entry) {
  atomicCAS(status, 0, code);
  if (bad) atomicMin(bad, entry);
}

// Exclusive scan of one int per thread across the block; returns the prefix
// and writes the block total.  `ws` needs blockDim.x/32 + 1 ints of shared
// memory.  All threads must call it.
template <int BLOCK>
__device__ __forceinline__ int block_exscan(int v, int* ws, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    constexpr int NW = BLOCK / 32;
    int s = lane < NW ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < NW) ws[lane] = s;  // inclusive per-warp totals
  }
  __syncthreads();
  int warp_off = wid ? ws[wid - 1] : 0;
  total = ws[BLOCK / 32 - 1];
  __syncthreads();
  return warp_off + x - v;
}

template <int BLOCK>
__device__ __forceinline__ long long block_sum_ll(long long v, long long* ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  long long t = 0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < BLOCK / 32; ++w) t += ws[w];
    ws[0] = t;
  }
  __syncthreads();
  t = ws[0];
  __syncthreads();
  return t;
}

template <int BLOCK>
__device__ __forceinline__ unsigned block_min_u32(unsigned v, unsigned* ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_down_sync(0xffffffffu, v, o));
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = ws[0];
    for (int w = 1; w < BLOCK / 32; ++w) t = min(t, ws[w]);
    ws[0] = t;
  }
  __syncthreads();
  unsigned r = ws[0];
  __syncthreads();
  return r;
}

template <int BLOCK>
__device__ __forceinline__ unsigned block_max_u32(unsigned v, unsigned* ws) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_down_sync(0xffffffffu, v, o));
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t = ws[0];
    for (int w = 1; w < BLOCK / 32; ++w) t = max(t, ws[w]);
    ws[0] = t;
  }
  __syncthreads();
  unsigned r = ws[0];
  __syncthreads();
  return r;
}

// Shared-memory workspace of the CTA radix sort.
template <int BLOCK>
struct SortSmem {
  unsigned offs[256];              // running digit offsets
  unsigned tot[256];               // digit counts of the current tile
  unsigned wcnt[BLOCK / 32][256];  // per-warp digit counts -> per-warp offsets
  unsigned ws[BLOCK / 32 + 1];
};

// Stable LSD radix sort (8-bit digits) of n keys by (key - kmin), done by one
// CTA.  `a` holds the input; `b` is scratch of the same size.  Both may live
// in shared or global memory (generic addressing).  Returns the buffer that
// holds the sorted keys.  All threads of the block must call it.
template <int BLOCK>
__device__ uint32_t* cta_radix_sort(uint32_t* a, uint32_t* b, int n, uint32_t kmin, int nbits,
                                    SortSmem<BLOCK>& sm) {
  static_assert(BLOCK >= 256 && BLOCK % 32 == 0, "BLOCK must cover the 256 digits");
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  constexpr int NW = BLOCK / 32;
  for (int shift = 0; shift < nbits; shift += 8) {
    if (tid < 256) {
      sm.offs[tid] = 0;
      for (int w = 0; w < NW; ++w) sm.wcnt[w][tid] = 0;
    }
    __syncthreads();
    for (int i = tid; i < n; i += BLOCK) atomicAdd(&sm.offs[((a[i] - kmin) >> shift) & 255u], 1u);
    __syncthreads();
    if (wid == 0) {  // exclusive scan of the 256 digit counts, 8 per lane
      unsigned v[8], s = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) { v[j] = sm.offs[lane * 8 + j]; s += v[j]; }
      unsigned x = s;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      unsigned run = x - s;
#pragma unroll
      for (int j = 0; j < 8; ++j) { sm.offs[lane * 8 + j] = run; run += v[j]; }
    }
    __syncthreads();
    // stable scatter, one tile of BLOCK keys at a time in input order
    for (int base = 0; base < n; base += BLOCK) {
      const int i = base + tid;
      const bool valid = i < n;
      const uint32_t key = valid ? a[i] : 0u;
      const unsigned d = valid ? (((key - kmin) >> shift) & 255u) : 256u;
      const unsigned peers = __match_any_sync(0xffffffffu, d);
      const unsigned rank = __popc(peers & lanemask_lt());
      if (valid && lane == __ffs(peers) - 1) sm.wcnt[wid][d] = __popc(peers);
      __syncthreads();
      if (tid < 256) {  // exclusive prefix over warps for digit tid
        unsigned run = 0;
        for (int w = 0; w < NW; ++w) {
          unsigned c = sm.wcnt[w][tid];
          sm.wcnt[w][tid] = run;
          run += c;
        }
        sm.tot[tid] = run;
      }
      __syncthreads();
      if (valid) b[sm.offs[d] + sm.wcnt[wid][d] + rank] = key;
      __syncthreads();
      if (tid < 256) {
        sm.offs[tid] += sm.tot[tid];
        for (int w = 0; w < NW; ++w) sm.wcnt[w][tid] = 0;
      }
      __syncthreads();
    }
    uint32_t* t = a;
    a = b;
    b = t;
  }
  return a;
}

}  // namespace sg
