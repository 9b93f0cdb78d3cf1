// Exact Euclidean k-nearest-neighbour graph, replacing the reference's
// kd-tree search (snapatac2-core/src/utils/knn.rs:9-31: squared Euclidean in
// FP64, self removed by index, first k kept, value = sqrt(distance); rows of
// the CSR sorted by column index, to_csr_matrix 58-78).
//
// Pipeline (no host synchronisation):
//  1. prep    X (n x d FP64) -> zero-padded FP32 and FP64 copies (n x DP),
//             max row norm.
//  2. scan    tiled brute force in FP32, filter then verify: a CTA owns 32
//             queries and streams 128-candidate tiles (stored tile-transposed,
//             so a tile is one coalesced 16 KB copy) through shared memory.
//             Filter: every thread computes 4 queries x 4 candidates in the
//             expanded form |q|^2 + |c|^2 - 2 q.c (one FFMA per dimension and
//             pair) and keeps the pairs that pass the current K'-th distance
//             tau widened by a bound on the FP32 error of that form (so no
//             pair whose exact-order difference-form distance is below tau is
//             dropped).  Verify: the warp recomputes the kept pairs in the
//             difference form sum (q_t - c_t)^2 (the FP32 arithmetic the
//             certificate below is stated for) and appends those below tau to
//             the query's list, re-sorted (warp bitonic) when it overflows.
//  3. rerank  FP64 distances of the K' candidates, sort by (distance, index),
//             keep k.  Certificate: every point outside the list has FP32
//             distance >= tau (the K'-th), hence FP64 distance >= tau - delta
//             with delta a bound on the FP32 error; if tau - delta > the k-th
//             FP64 distance the FP64 top-k is exact, otherwise the query is
//             queued for
//  4. exact   the same scan in FP64 for the queued queries only.
//  5. rows sorted by column index, distances sqrt'ed.
// Ties are broken by the smaller index.
#include <cuda_bf16.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>

#include <type_traits>

#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kQT = 32;    // queries per CTA (one per lane)
constexpr int kCT = 128;   // candidates per shared-memory tile
constexpr int kLW = 8;     // warps per CTA
constexpr int kList = 256; // per-query list + append buffer
constexpr int kMaxKp = 128;

template <typename K>
__device__ __forceinline__ bool lex_gt(K a, int ia, K b, int ib) {
  return a > b || (a == b && ia > ib);
}

// Ascending bitonic sort of N = 2^p (key, idx) pairs in shared memory by one warp.
template <typename K>
__device__ void warp_bitonic(K* key, int* idx, int N) {
  const int lane = threadIdx.x & 31;
  for (int size = 2; size <= N; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < (N >> 1); t += 32) {
        const int i = 2 * t - (t & (stride - 1));
        const int j = i + stride;
        const bool asc = (i & size) == 0;
        const K ki = key[i], kj = key[j];
        const int ii = idx[i], ij = idx[j];
        if (lex_gt(ki, ii, kj, ij) == asc) {
          key[i] = kj; key[j] = ki;
          idx[i] = ij; idx[j] = ii;
        }
      }
      __syncwarp();
    }
  }
}

template <typename K> __device__ __forceinline__ K kinf();
template <> __device__ __forceinline__ double kinf<double>() { return DBL_MAX; }

template <typename TD, int DP>
struct ScanSmem {
  TD cv[kCT][DP];          // candidate tile
  TD dist[kQT][kCT + 1];   // distance tile
  TD lk[kQT][kList];       // per-query list keys
  int li[kQT][kList];      // per-query list indices
  int cnt[kQT];
  TD tau[kQT];
};

// Sort query q's list (warp), keep Kp, update tau.
template <typename TD, int DP>
__device__ void merge_list(ScanSmem<TD, DP>& sm, int q, int Kp) {
  const int lane = threadIdx.x & 31;
  const int c = sm.cnt[q];
  for (int t = c + lane; t < kList; t += 32) {
    sm.lk[q][t] = kinf<TD>();
    sm.li[q][t] = 0x7fffffff;
  }
  __syncwarp();
  warp_bitonic<TD>(sm.lk[q], sm.li[q], kList);
  __syncwarp();
  if (lane == 0) {
    const int keep = c < Kp ? c : Kp;
    sm.cnt[q] = keep;
    sm.tau[q] = keep == Kp ? sm.lk[q][Kp - 1] : kinf<TD>();
  }
  __syncwarp();
}

// Scan all n points for queries qlist[blockIdx.x*32 + lane] (or the identity
// when qlist == nullptr).  Writes per query the Kp best (distance, index)
// sorted ascending, and tau = Kp-th distance (inf if fewer).
template <typename TD, int DP>
__global__ void __launch_bounds__(kLW * 32)
scan_kernel(const TD* __restrict__ Xp, int64_t n, const int* __restrict__ qlist, const int* __restrict__ qcount,
            int Kp, int* __restrict__ cand, TD* __restrict__ cand_d, TD* __restrict__ tau_out) {
  extern __shared__ __align__(128) unsigned char sraw[];
  ScanSmem<TD, DP>& sm = *reinterpret_cast<ScanSmem<TD, DP>*>(sraw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t nq = qcount ? (int64_t)*qcount : n;
  const int64_t qbase = (int64_t)blockIdx.x * kQT;
  if (qbase >= nq) return;  // uniform across the CTA
  const int64_t qslot = qbase + lane;
  const bool qvalid = qslot < nq;
  const int64_t qid = qvalid ? (qlist ? (int64_t)qlist[qslot] : qslot) : -1;

  using V = typename std::conditional<sizeof(TD) == 4, float4, double2>::type;
  constexpr int VW = 16 / sizeof(TD);
  TD qr[DP];
#pragma unroll
  for (int t = 0; t < DP; t += VW) {
    V v;
    if (qvalid) v = *reinterpret_cast<const V*>(Xp + qid * DP + t);
    else memset(&v, 0, sizeof(v));
    const TD* pv = reinterpret_cast<const TD*>(&v);
#pragma unroll
    for (int s = 0; s < VW; ++s) qr[t + s] = pv[s];
  }
  if (threadIdx.x < kQT) {
    sm.cnt[threadIdx.x] = 0;
    sm.tau[threadIdx.x] = kinf<TD>();
  }
  for (int64_t c0 = 0; c0 < n; c0 += kCT) {
    __syncthreads();
    // load candidate tile
    const int nct = (n - c0) < kCT ? (int)(n - c0) : kCT;
    for (int t = threadIdx.x; t < kCT * DP / VW; t += kLW * 32) {
      const int r = t / (DP / VW), v = t % (DP / VW);
      V val;
      if (r < nct) val = *reinterpret_cast<const V*>(Xp + (c0 + r) * DP + v * VW);
      else memset(&val, 0, sizeof(val));
      *reinterpret_cast<V*>(&sm.cv[r][v * VW]) = val;
    }
    __syncthreads();
    // distances: lane = query, warp covers candidates wid, wid+8, ...
#pragma unroll 2
    for (int j = 0; j < kCT / kLW; ++j) {
      const int c = wid + j * kLW;
      TD acc = TD(0);
#pragma unroll
      for (int t = 0; t < DP; t += VW) {
        const V v = *reinterpret_cast<const V*>(&sm.cv[c][t]);
        const TD* pv = reinterpret_cast<const TD*>(&v);
#pragma unroll
        for (int s = 0; s < VW; ++s) {
          if (sizeof(TD) == 8) {  // FP64 pass: the reference's unfused arithmetic
            const double df = __dsub_rn((double)qr[t + s], (double)pv[s]);
            acc = (TD)__dadd_rn((double)acc, __dmul_rn(df, df));
          } else {
            const TD df = qr[t + s] - pv[s];
            acc = fma(df, df, acc);
          }
        }
      }
      const int64_t cg = c0 + c;
      if (c >= nct || cg == qid || !qvalid) acc = kinf<TD>();
      sm.dist[lane][c] = acc;
    }
    __syncthreads();
    // fused selection: warp wid owns queries 4*wid .. 4*wid+3
    for (int qq = 0; qq < kQT / kLW; ++qq) {
      const int q = wid * (kQT / kLW) + qq;
      const TD th = sm.tau[q];
      int base = sm.cnt[q];
#pragma unroll
      for (int j = 0; j < kCT / 32; ++j) {
        const int c = lane + 32 * j;
        const TD dv = sm.dist[q][c];
        const bool take = dv < th;
        const unsigned bal = __ballot_sync(0xffffffffu, take);
        if (take) {
          const int p = base + __popc(bal & lanemask_lt());
          sm.lk[q][p] = dv;
          sm.li[q][p] = (int)(c0 + c);
        }
        base += __popc(bal);
      }
      __syncwarp();
      if (lane == 0) sm.cnt[q] = base;
      __syncwarp();
      if (base > kList - kCT) merge_list<TD, DP>(sm, q, Kp);
    }
  }
  __syncthreads();
  for (int qq = 0; qq < kQT / kLW; ++qq) {
    const int q = wid * (kQT / kLW) + qq;
    merge_list<TD, DP>(sm, q, Kp);
    const int64_t qs = qbase + q;
    if (qs < nq) {
      const int c = sm.cnt[q];
      for (int t = lane; t < Kp; t += 32) {
        cand[qs * Kp + t] = t < c ? sm.li[q][t] : -1;
        if (cand_d) cand_d[qs * Kp + t] = t < c ? sm.lk[q][t] : kinf<TD>();
      }
      if (lane == 0 && tau_out) tau_out[qs] = sm.tau[q];
    }
  }
}

// ---------------------------------------------------------------------------
// FP32 filter-verify scan (step 2).  XT holds the centred FP32 points tile-
// transposed: tile t (points 128t .. 128t+127) at XT + t*DP*128, coordinate
// (dim, j) at [dim*128 + j], zero beyond n; nrm[i] = FP32 of |x_i - mean|^2.
// ---------------------------------------------------------------------------
constexpr int kFQ = 32;          // queries per CTA
constexpr int kFC = 128;         // candidates per tile
constexpr int kFW = 8;           // warps per CTA (warp w owns queries 4w .. 4w+3)
constexpr int kFBuf = 3;         // candidate tiles in flight (ring)

// LIST entries per query: the kept Kp plus one verify batch of 32 (a list is
// re-sorted before a batch that would not fit), so LIST >= Kp + 32.
template <int DP, int LIST>
struct FilterSmem {
  uint64_t full[kFBuf];                      // tile k landed in buffer k % kFBuf
  uint64_t empty[kFBuf];                     // every warp is done with that buffer
  __align__(16) float cT[kFBuf][DP][kFC];    // candidate tiles (bulk copies of XT)
  __align__(16) float cn[kFBuf][kFC];        // their squared norms (bulk copies of nrm)
  __align__(16) float qT[DP][kFQ];
  float lk[kFQ][LIST];
  int li[kFQ][LIST];
  int cnt[kFQ];
  float tau[kFQ];
  unsigned queue[kFW][kFC];                  // one query's filtered candidates of a tile
  int nqueue[kFW];
};

// Sort one query's list (warp), keep Kp, update its tau.
template <int LIST>
__device__ void merge_list_f(float* lk, int* li, int* cnt, float* tau, int Kp) {
  const int lane = threadIdx.x & 31;
  const int c = *cnt;
  for (int t = c + lane; t < LIST; t += 32) {
    lk[t] = FLT_MAX;
    li[t] = 0x7fffffff;
  }
  __syncwarp();
  warp_bitonic<float>(lk, li, LIST);
  __syncwarp();
  if (lane == 0) {
    const int keep = c < Kp ? c : Kp;
    *cnt = keep;
    *tau = keep == Kp ? lk[Kp - 1] : FLT_MAX;
  }
  __syncwarp();
}

// Warps advance through the tiles on their own: a tile is consumed once its
// copy lands (full barrier), and its buffer is refilled only after all
// warps arrived on its empty barrier, so a warp busy re-sorting a list holds
// up the others only once they run a whole ring ahead.  Thread 0 produces.
template <int DP, int LIST>
__global__ void __launch_bounds__(kFW * 32, 2)
filter_scan_kernel(const float* __restrict__ XT, const float* __restrict__ nrm, int64_t n, int d, int Kp,
                   int* __restrict__ cand, float* __restrict__ tau_out) {
  extern __shared__ __align__(128) unsigned char sraw[];
  FilterSmem<DP, LIST>& sm = *reinterpret_cast<FilterSmem<DP, LIST>*>(sraw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t qbase = (int64_t)blockIdx.x * kFQ;
  const int64_t ntiles = (n + kFC - 1) / kFC;
  constexpr uint32_t kTileBytes = DP * kFC * 4, kNormBytes = kFC * 4;
  auto issue = [&](int64_t k) {
    const int b = (int)(k % kFBuf);
    mbar_expect_tx(&sm.full[b], kTileBytes + kNormBytes);
    bulk_copy(&sm.cT[b][0][0], XT + k * DP * kFC, kTileBytes, &sm.full[b]);
    bulk_copy(&sm.cn[b][0], nrm + k * kFC, kNormBytes, &sm.full[b]);
  };
  if (threadIdx.x == 0) {
    for (int b = 0; b < kFBuf; ++b) {
      mbar_init(&sm.full[b], 1);
      mbar_init(&sm.empty[b], kFW);
    }
    fence_barrier_init();
    fence_proxy_async();
    for (int64_t k = 0; k < kFBuf - 1 && k < ntiles; ++k) issue(k);
  }
  {
    const float* src = XT + (qbase / kFC) * DP * kFC + (qbase % kFC);
    for (int e = threadIdx.x; e < DP * kFQ; e += blockDim.x) sm.qT[e / kFQ][e % kFQ] = src[(e / kFQ) * kFC + e % kFQ];
  }
  if (threadIdx.x < kFQ) {
    sm.cnt[threadIdx.x] = 0;
    sm.tau[threadIdx.x] = FLT_MAX;
  }
  if (lane == 0) sm.nqueue[wid] = 0;
  float qn[4];
  int64_t qid[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    qid[i] = qbase + 4 * wid + i;
    qn[i] = qid[i] < n ? nrm[qid[i]] : 0.f;
  }
  __syncthreads();
  // Filter bound.  With u = 2^-24, s the FP32 dot product (FMA chain over DP
  // terms), nq, nc the FP32 squared norms and D^ the exact squared distance
  // of the FP32 points: |(nq + nc - 2 s) - D^| <= (DP + 3) u (nq + nc) + u D^,
  // and the difference-form FP32 distance d32 obeys |d32 - D^| <= (d + 3) u D^.
  // So d32 < tau implies nq + nc - 2 s < tau + Ku (nq + nc) + Tu tau with
  // K = 2 DP + 16, T = 4 (d + 4) (twice the derived constants, which also
  // covers the rounding of the test itself), written as
  // nc (1 - Ku) - 2 s < tau (1 + Tu) + Ku nq - nq.
  const float u = 5.9604644775390625e-08f;
  const float Ku = (float)(2 * DP + 16) * u, Tu = (float)(4 * (d + 4)) * u;
  const float kInf = __int_as_float(0x7f800000);
  bool failed = false;
  int64_t issued = kFBuf - 1 < ntiles ? kFBuf - 1 : ntiles;  // tiles handed to the copy engine (thread 0)
  for (int64_t k = 0; k < ntiles; ++k) {
    const int b = (int)(k % kFBuf);
    bool pfail = false;
    if (threadIdx.x == 0 && k + kFBuf - 1 < ntiles) {
      // refill the buffer tile k - 1 used, once every warp is done with it
      const int64_t kn = k + kFBuf - 1;
      const bool ok = kn < kFBuf || mbar_wait(&sm.empty[kn % kFBuf], (uint32_t)(((kn / kFBuf) - 1) & 1));
      if (ok) {
        fence_proxy_async();
        issue(kn);
        issued = kn + 1;
      } else {
        pfail = true;
      }
    }
    const bool got = !pfail && mbar_wait(&sm.full[b], (uint32_t)((k / kFBuf) & 1));
    if (!__all_sync(0xffffffffu, got)) {
      failed = true;  // a tile never landed: leave this warp's queries to the exact rescan
      break;
    }
    const int64_t c0 = k * kFC;
    float T[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float tq = sm.tau[4 * wid + i];
      T[i] = qid[i] >= n ? -kInf : (tq >= FLT_MAX ? kInf : (tq + Tu * tq) + (Ku * qn[i] - qn[i]));
    }
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
#pragma unroll 8
    for (int t = 0; t < DP; ++t) {
      const float4 qv = *reinterpret_cast<const float4*>(&sm.qT[t][4 * wid]);
      const float4 cv = *reinterpret_cast<const float4*>(&sm.cT[b][t][4 * lane]);
      const float qa[4] = {qv.x, qv.y, qv.z, qv.w}, ca[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(qa[i], ca[j], acc[i][j]);
    }
    const float4 cn4 = *reinterpret_cast<const float4*>(&sm.cn[b][4 * lane]);
    const float cadj[4] = {cn4.x * (1.0f - Ku), cn4.y * (1.0f - Ku), cn4.z * (1.0f - Ku), cn4.w * (1.0f - Ku)};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int q = 4 * wid + i;
      const int64_t so = qid[i] - c0;  // the query's own column in this tile, if any
      const int self = (so >= 0 && so < kFC) ? (int)so : -1;
      bool keep[4];
      bool any = false;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        keep[j] = fmaf(-2.0f, acc[i][j], cadj[j]) < T[i] && 4 * lane + j != self;
        any |= keep[j];
      }
      if (!__any_sync(0xffffffffu, any)) continue;  // nothing of this query passed the filter
#pragma unroll
      for (int j = 0; j < 4; ++j)
        if (keep[j]) sm.queue[wid][atomicAdd(&sm.nqueue[wid], 1)] = (unsigned)(4 * lane + j);
      __syncwarp();
      // verify in the difference form; append (ballot order) those below tau,
      // re-sorting the list first when the batch would not fit
      const int nk = sm.nqueue[wid];
      int cq = sm.cnt[q];
      for (int e0 = 0; e0 < nk; e0 += 32) {
        const int e = e0 + lane;
        int c = 0;
        float dd = kInf;
        if (e < nk) {
          c = (int)sm.queue[wid][e];
          dd = 0.f;
#pragma unroll
          for (int t = 0; t < DP; ++t) {
            const float df = sm.qT[t][q] - sm.cT[b][t][c];
            dd = fmaf(df, df, dd);
          }
        }
        bool pass = dd < sm.tau[q];
        unsigned bal = __ballot_sync(0xffffffffu, pass);
        if (cq + __popc(bal) > LIST) {
          if (lane == 0) sm.cnt[q] = cq;
          __syncwarp();
          merge_list_f<LIST>(sm.lk[q], sm.li[q], &sm.cnt[q], &sm.tau[q], Kp);
          cq = sm.cnt[q];
          pass = dd < sm.tau[q];
          bal = __ballot_sync(0xffffffffu, pass);
        }
        if (pass) {
          const int p = cq + __popc(bal & lanemask_lt());
          sm.lk[q][p] = dd;
          sm.li[q][p] = (int)(c0 + c);
        }
        cq += __popc(bal);
      }
      if (lane == 0) {
        sm.cnt[q] = cq;
        sm.nqueue[wid] = 0;
      }
      __syncwarp();
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&sm.empty[b]);  // this warp is done with buffer b
  }
  failed = __any_sync(0xffffffffu, failed);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int q = 4 * wid + i;
    if (!failed) merge_list_f<LIST>(sm.lk[q], sm.li[q], &sm.cnt[q], &sm.tau[q], Kp);
    if (qid[i] < n) {
      const int c = failed ? 0 : sm.cnt[q];
      for (int t = lane; t < Kp; t += 32) cand[qid[i] * Kp + t] = t < c ? sm.li[q][t] : -1;
      if (lane == 0) tau_out[qid[i]] = failed ? -1.0f : sm.tau[q];  // negative tau: certificate fails
    }
  }
  // no copy may still be landing in this CTA's shared memory when it exits:
  // after a failure, wait (bounded) for the last tiles thread 0 issued
  if (threadIdx.x == 0 && failed)
    for (int64_t t = issued - kFBuf < 0 ? 0 : issued - kFBuf; t < issued; ++t)
      mbar_wait(&sm.full[t % kFBuf], (uint32_t)((t / kFBuf) & 1));
}

// ---------------------------------------------------------------------------
// Tensor-core filter (d <= 32).  The filter's dot products q.c come from
// tcgen05.mma: the centred FP32 coordinates are split into bf16 hi + lo and
// q.c ~= qh.ch + qh.cl + ql.ch (three K = 32 products per 128 x 128 tile,
// FP32 accumulation in TMEM).  Dropped terms and accumulation stay below
// 6e-5 sum|q_t c_t|; the filter is widened by KTC = 2^-12 of nq + nc (four
// times that), so, as in the FP32 filter, no pair whose difference-form
// distance is below tau is dropped; the verify, the lists and the output are
// those of filter_scan_kernel.
//
// TC layout (prep): per 128-point tile, [hi 8 KB][lo 8 KB][lo2 8 KB]
// [nc (1 - K) 512 B], each bf16 array in the no-swizzle K-major core-matrix
// layout: element (row r, dim t) at byte (r/8)*512 + (t/8)*128 + (r%8)*16 +
// (t%8)*2.  hi = RN(v), lo = RN(v - hi), lo2 = RN(v - hi - lo) (bf16): the
// remainders have at most 16 and 8 significant bits, so hi + lo + lo2 == v
// exactly and the verify reads exact FP32 coordinates from shared memory.
// ---------------------------------------------------------------------------
constexpr int kTQ = 128;                  // queries per CTA (MMA M)
constexpr int kTC = 128;                  // candidates per tile (MMA N)
constexpr int kTDim = 32;                 // K (padded dimensions)
constexpr int kTMat = kTQ * kTDim * 2;    // one bf16 operand: 8 KB
constexpr int kTTile = 3 * kTMat + kTC * 4;  // hi, lo, lo2, scaled norms
constexpr int kTBuf = 2;
constexpr int kTList = 128;               // Kp + 16 <= 128
constexpr int kTChunk = 16;               // candidates per thread between verify rounds
constexpr int kTQueue = 32 * kTChunk;     // per consumer warp
constexpr int kTConsumers = 4;            // warps 0..3 read TMEM lanes 32w..32w+31
constexpr int kTThreads = (kTConsumers + 1) * 32;  // + one producer warp
constexpr float kTcK = 2.44140625e-4f + 8.0f * 5.9604644775390625e-08f;  // 2^-12 + rounding of the test

struct TcSmem {
  uint64_t full[kTBuf];     // tile landed
  uint64_t sfree[kTBuf];    // tile consumed: MMA done (commit) + 4 consumer warps
  uint64_t mdone[2];        // accumulator buffer x holds tile k (commit)
  uint64_t tfree[2];        // accumulator buffer x read by the 4 consumer warps
  uint64_t aful;            // query operands landed
  uint64_t drain;           // failure path: every MMA issued so far has completed (commit)
  uint32_t tmem_slot;
  int failed;
  __align__(128) unsigned char A[2 * kTMat];
  __align__(128) unsigned char Bt[kTBuf][kTTile];
  float qT[kTDim][kTQ];
  float lk[kTQ][kTList];
  int li[kTQ][kTList];
  int cnt[kTQ];
  float tau[kTQ];
  unsigned queue[kTConsumers][kTQueue];
  int nqueue[kTConsumers];
};

static_assert(sizeof(TcSmem) <= 232448, "tensor-core filter shared memory above the per-CTA limit");

__device__ __forceinline__ uint32_t tc_off(int r, int t) {
  return (uint32_t)((r >> 3) * 512 + (t >> 3) * 128 + (r & 7) * 16 + (t & 7) * 2);
}

// TC layout from the tile-transposed FP32 copy (XT) and the norms.
__global__ void tc_prep_kernel(const float* __restrict__ XT, const float* __restrict__ nrm, int64_t n,
                               unsigned char* __restrict__ TC) {
  const int64_t npad = (n + kFC - 1) / kFC * kFC;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i / kFC;
    const int r = (int)(i % kFC);
    unsigned char* tile = TC + k * kTTile;
    const float* src = XT + k * 32 * kFC + r;
    for (int t = 0; t < kTDim; ++t) {
      const float v = src[t * kFC];
      const __nv_bfloat16 h = __float2bfloat16_rn(v);
      const float r1 = v - __bfloat162float(h);
      const __nv_bfloat16 l = __float2bfloat16_rn(r1);
      const __nv_bfloat16 l2 = __float2bfloat16_rn(r1 - __bfloat162float(l));
      *reinterpret_cast<__nv_bfloat16*>(tile + tc_off(r, t)) = h;
      *reinterpret_cast<__nv_bfloat16*>(tile + kTMat + tc_off(r, t)) = l;
      *reinterpret_cast<__nv_bfloat16*>(tile + 2 * kTMat + tc_off(r, t)) = l2;
    }
    reinterpret_cast<float*>(tile + 3 * kTMat)[r] = nrm[i] * (1.0f - kTcK);  // the filter's nc (1 - K)
  }
}

__global__ void __launch_bounds__(kTThreads, 1)
tc_filter_kernel(const float* __restrict__ XT, const unsigned char* __restrict__ TC, const float* __restrict__ nrm,
                 int64_t n, int d, int Kp, int* __restrict__ cand, float* __restrict__ tau_out) {
  extern __shared__ __align__(128) unsigned char sraw[];
  TcSmem& sm = *reinterpret_cast<TcSmem*>(sraw);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t qbase = (int64_t)blockIdx.x * kTQ;
  const int64_t ntiles = (n + kTC - 1) / kTC;
  if (wid == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&sm.tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    for (int b = 0; b < kTBuf; ++b) {
      mbar_init(&sm.full[b], 1);
      mbar_init(&sm.sfree[b], 1 + kTConsumers);
    }
    for (int x = 0; x < 2; ++x) {
      mbar_init(&sm.mdone[x], 1);
      mbar_init(&sm.tfree[x], kTConsumers);
    }
    mbar_init(&sm.aful, 1);
    mbar_init(&sm.drain, 1);
    sm.failed = 0;
    fence_barrier_init();
  }
  if (wid < kTConsumers) {
    const float* src = XT + (qbase / kFC) * 32 * kFC;
    for (int e = threadIdx.x; e < kTDim * kTQ; e += kTConsumers * 32) sm.qT[e / kTQ][e % kTQ] = src[e];
    if (lane < 32) {
      sm.cnt[wid * 32 + lane] = 0;
      sm.tau[wid * 32 + lane] = FLT_MAX;
    }
    if (lane == 0) sm.nqueue[wid] = 0;
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = sm.tmem_slot;
  const uint32_t idesc = umma_idesc_bf16(kTQ, kTC);
  bool failed = false;

  if (wid == kTConsumers) {
    // ---------------- producer: tile copies and MMAs (one thread) ---------
    if (lane == 0) {
      // tiles [waited, issued) have copies in flight, at most one per buffer
      int64_t issued = 0, waited = 0;
      auto issue = [&](int64_t k) {
        const int b = (int)(k % kTBuf);
        mbar_expect_tx(&sm.full[b], kTTile);
        bulk_copy(sm.Bt[b], TC + k * kTTile, kTTile, &sm.full[b]);
        issued = k + 1;
      };
      mbar_expect_tx(&sm.aful, 2 * kTMat);
      bulk_copy(sm.A, TC + (qbase / kFC) * kTTile, 2 * kTMat, &sm.aful);
      for (int64_t k = 0; k < kTBuf && k < ntiles; ++k) issue(k);
      const bool a_ok = mbar_wait(&sm.aful, 0);
      bool ok = a_ok;
      const uint32_t a_hi = smem_u32(sm.A), a_lo = a_hi + kTMat;
      // tile k: MMA as soon as it landed and its accumulator buffer was read
      // out (tile k - 2); then refill the buffer tile k - 1 used with tile
      // k + 1 once the consumers are done with tile k - 1: the copy and the
      // tensor cores work on tile k + 1 while the consumers filter tile k.
      for (int64_t k = 0; ok && k < ntiles; ++k) {
        const int b = (int)(k % kTBuf), x = (int)(k & 1);
        ok = mbar_wait(&sm.full[b], (uint32_t)((k / kTBuf) & 1));
        if (ok) waited = k + 1;
        if (ok && k >= 2) ok = mbar_wait(&sm.tfree[x], (uint32_t)(((k / 2) - 1) & 1));
        if (!ok) break;
        tc_fence_after();
        const uint32_t b_hi = smem_u32(sm.Bt[b]), b_lo = b_hi + kTMat;
        const uint32_t dst = tmem + (uint32_t)(x * kTC);
        const uint32_t pa[3] = {a_hi, a_hi, a_lo}, pb[3] = {b_hi, b_lo, b_hi};
#pragma unroll
        for (int p = 0; p < 3; ++p)
#pragma unroll
          for (int ks = 0; ks < kTDim / 16; ++ks)
            umma_bf16(dst, umma_desc(pa[p] + ks * 256u, 128u, 512u), umma_desc(pb[p] + ks * 256u, 128u, 512u), idesc,
                      p > 0 || ks > 0);
        umma_commit(&sm.mdone[x]);
        umma_commit(&sm.sfree[b]);
        const int64_t kt = k + kTBuf - 1;  // into the buffer tile k - 1 used
        if (kt < ntiles && kt >= kTBuf) {
          ok = mbar_wait(&sm.sfree[(k - 1) % kTBuf], (uint32_t)(((k - 1) / kTBuf) & 1));
          if (!ok) break;
          fence_proxy_async();
          issue(kt);
        }
      }
      if (!ok) {
        atomicExch(&sm.failed, 1);
        // before the CTA frees TMEM and exits, let what is in flight land:
        // the query copy, every tile copy not yet waited for (one phase per
        // buffer, so each parity wait is unambiguous) and every committed
        // MMA (a last commit completes once all earlier ones have); each
        // wait is bounded like the others
        if (!a_ok) mbar_wait(&sm.aful, 0);
        for (int64_t t = waited; t < issued; ++t) mbar_wait(&sm.full[t % kTBuf], (uint32_t)((t / kTBuf) & 1));
        umma_commit(&sm.drain);
        mbar_wait(&sm.drain, 0);
      }
    }
  } else {
    // ---------------- consumers: filter from TMEM, verify, lists ----------
    const int row = wid * 32 + lane;
    const int64_t q = qbase + row;
    const float nq = q < n ? nrm[q] : 0.f;
    const float u = 5.9604644775390625e-08f;
    const float Tu = (float)(4 * (d + 4)) * u;
    const float kInf = __int_as_float(0x7f800000);
    for (int64_t k = 0; k < ntiles; ++k) {
      const int b = (int)(k % kTBuf), x = (int)(k & 1);
      bool ok = mbar_wait(&sm.mdone[x], (uint32_t)((k / 2) & 1));
      ok = ok && mbar_wait(&sm.full[b], (uint32_t)((k / kTBuf) & 1));  // the norms of this tile
      if (!__all_sync(0xffffffffu, ok)) {
        failed = true;
        break;
      }
      tc_fence_after();
      const int64_t c0 = k * kTC;
      const float4* cadj4 = reinterpret_cast<const float4*>(sm.Bt[b] + 3 * kTMat);
      const float tq = sm.tau[row];
      const float T = q >= n ? -kInf : (tq >= FLT_MAX ? kInf : (tq + Tu * tq) + (kTcK * nq - nq));
      // acceptance masks, 32 candidates (one TMEM load) at a time; the
      // query's own column is removed in the verify step
      uint32_t mw[4];
#pragma unroll
      for (int w4 = 0; w4 < 4; ++w4) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(wid * 32) << 16) + (uint32_t)(x * kTC + 32 * w4), v);
        uint32_t mm = 0;
#pragma unroll
        for (int j4 = 0; j4 < 8; ++j4) {
          const float4 c = cadj4[8 * w4 + j4];
          mm |= (fmaf(-2.0f, v[4 * j4 + 0], c.x) < T ? 1u : 0u) << (4 * j4 + 0);
          mm |= (fmaf(-2.0f, v[4 * j4 + 1], c.y) < T ? 1u : 0u) << (4 * j4 + 1);
          mm |= (fmaf(-2.0f, v[4 * j4 + 2], c.z) < T ? 1u : 0u) << (4 * j4 + 2);
          mm |= (fmaf(-2.0f, v[4 * j4 + 3], c.w) < T ? 1u : 0u) << (4 * j4 + 3);
        }
        mw[w4] = mm;
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.tfree[x]);  // accumulator buffer x may be overwritten
      uint32_t m0 = mw[0], m1 = mw[1], m2 = mw[2], m3 = mw[3];
      // drain the masks in rounds of at most kTChunk pairs per lane
#pragma unroll 1
      while (__any_sync(0xffffffffu, (m0 | m1 | m2 | m3) != 0)) {
        int mine = 0;
#pragma unroll 1
        while (mine < kTChunk && (m0 | m1 | m2 | m3)) {
          int j;
          if (m0) { j = __ffs(m0) - 1; m0 &= m0 - 1; }
          else if (m1) { j = 32 + __ffs(m1) - 1; m1 &= m1 - 1; }
          else if (m2) { j = 64 + __ffs(m2) - 1; m2 &= m2 - 1; }
          else { j = 96 + __ffs(m3) - 1; m3 &= m3 - 1; }
          sm.queue[wid][atomicAdd(&sm.nqueue[wid], 1)] = ((unsigned)lane << 16) | (unsigned)j;
          ++mine;
        }
        // make room: re-sort the lists that this round could overflow
        unsigned need = __ballot_sync(0xffffffffu, sm.cnt[row] + mine > kTList);
        while (need) {
          const int l = __ffs(need) - 1;
          need &= need - 1;
          const int r = wid * 32 + l;
          merge_list_f<kTList>(sm.lk[r], sm.li[r], &sm.cnt[r], &sm.tau[r], Kp);
        }
        __syncwarp();
        const int nk = sm.nqueue[wid];
        for (int e = lane; e < nk; e += 32) {
          const unsigned pr = sm.queue[wid][e];
          const int r = wid * 32 + (int)(pr >> 16), c = (int)(pr & 0xffffu);
          if (c0 + c == qbase + r) continue;  // the query itself
          const unsigned char* tb = sm.Bt[b];
          float dd = 0.f;
#pragma unroll
          for (int t = 0; t < kTDim; ++t) {
            const uint32_t o = tc_off(c, t);
            const float cv = (__bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(tb + o)) +
                              __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(tb + kTMat + o))) +
                             __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(tb + 2 * kTMat + o));
            const float df = sm.qT[t][r] - cv;
            dd = fmaf(df, df, dd);
          }
          if (dd < sm.tau[r]) {
            const int p = atomicAdd(&sm.cnt[r], 1);
            sm.lk[r][p] = dd;
            sm.li[r][p] = (int)(c0 + c);
          }
        }
        __syncwarp();
        if (lane == 0) sm.nqueue[wid] = 0;
        __syncwarp();
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&sm.sfree[b]);  // done with this tile's norms
    }
    failed = __any_sync(0xffffffffu, failed);
    for (int l = 0; l < 32; ++l) {
      const int r = wid * 32 + l;
      const int64_t qq = qbase + r;
      if (!failed) merge_list_f<kTList>(sm.lk[r], sm.li[r], &sm.cnt[r], &sm.tau[r], Kp);
      if (qq < n) {
        const int c = failed ? 0 : sm.cnt[r];
        for (int t = lane; t < Kp; t += 32) cand[qq * Kp + t] = t < c ? sm.li[r][t] : -1;
        if (lane == 0) tau_out[qq] = failed ? -1.0f : sm.tau[r];  // negative tau: certificate fails
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  // a producer failure leaves every consumer result to the exact rescan
  if (sm.failed && wid < kTConsumers) {
    for (int l = 0; l < 32; ++l) {
      const int64_t qq = qbase + wid * 32 + l;
      if (qq < n && lane == 0) tau_out[qq] = -1.0f;
    }
  }
  tc_fence_after();
  if (wid == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tmem));
}

constexpr int kMeanParts = 256;

// Column means of X (n x d FP64), deterministic: per-CTA partial sums, then a
// fixed-order reduction.  The FP32 copy is centred on them, which removes the
// component every point shares and shrinks the FP32 rounding of distances.
__global__ void mean_partial(const double* __restrict__ X, int64_t n, int d, double* __restrict__ part) {
  const int b = blockIdx.x, nb = gridDim.x;
  const int64_t r0 = n * b / nb, r1 = n * (b + 1) / nb;
  for (int t = threadIdx.x; t < d; t += blockDim.x) {
    double s = 0.0;
    for (int64_t i = r0; i < r1; ++i) s += X[i * d + t];
    part[b * 64 + t] = s;
  }
}

__global__ void mean_reduce(const double* __restrict__ part, int nparts, int64_t n, int d, double* __restrict__ mean) {
  const int t = threadIdx.x;
  if (t >= 64) return;
  double s = 0.0;
  if (t < d)
    for (int b = 0; b < nparts; ++b) s += part[b * 64 + t];
  mean[t] = t < d ? s / (double)n : 0.0;
}

// X -> centred FP32 copy, tile-transposed for the filter scan (XT, zero
// beyond n up to the tile boundary), its FP32 squared norms, the padded FP64
// copy (uncentred: the re-rank uses the reference's arithmetic on the
// original coordinates) and the max centred row norm (float bits, rounded up).
template <int DP>
__global__ void prep_kernel(const double* __restrict__ X, int64_t n, int d, const double* __restrict__ mean,
                            float* __restrict__ XT, float* __restrict__ nrm, double* __restrict__ X64,
                            unsigned* __restrict__ maxnorm_bits) {
  float mx = 0.f;
  const int64_t npad = (n + kFC - 1) / kFC * kFC;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x) {
    float* dst = XT + (i / kFC) * DP * kFC + (i % kFC);
    if (i >= n) {
      for (int t = 0; t < DP; ++t) dst[t * kFC] = 0.f;
      nrm[i] = __int_as_float(0x7f800000);  // never passes the filter
      continue;
    }
    double s = 0.0, s32 = 0.0;
#pragma unroll 4
    for (int t = 0; t < DP; ++t) {
      const double v = t < d ? X[i * d + t] : 0.0;
      const double c = t < d ? v - mean[t] : 0.0;
      const float c32 = (float)c;
      dst[t * kFC] = c32;
      X64[i * DP + t] = v;
      s += c * c;
      s32 += (double)c32 * (double)c32;
    }
    nrm[i] = (float)s32;
    mx = fmaxf(mx, (float)sqrt(s) * 1.0000002f);
  }
  for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((threadIdx.x & 31) == 0) atomicMax(maxnorm_bits, __float_as_uint(mx));
}

// Write row q: the k (distance, index) pairs in kd[0..k) / ki[0..k) (any
// order) sorted by column index, distances sqrt'ed.  Uses kk/ks scratch.
__device__ void emit_row(int64_t q, int k, const double* kd, const int* kidx, double* kk, int* ks,
                         int64_t* __restrict__ nbr, double* __restrict__ dist) {
  const int lane = threadIdx.x & 31;
  for (int s = lane; s < kMaxKp; s += 32) {
    kk[s] = s < k ? (double)kidx[s] : DBL_MAX;
    ks[s] = s < k ? s : 0x7fffffff;
  }
  __syncwarp();
  warp_bitonic<double>(kk, ks, kMaxKp);
  for (int t = lane; t < k; t += 32) {
    nbr[q * k + t] = (int64_t)kk[t];
    dist[q * k + t] = sqrt(kd[ks[t]]);
  }
  __syncwarp();
}

// FP64 re-rank of the Kp FP32 candidates (warp per query), certificate check.
template <int DP>
__global__ void __launch_bounds__(256)
rerank_kernel(const double* __restrict__ X64, int64_t n, int d, const double* __restrict__ mean,
              const int* __restrict__ cand, int Kp, const float* __restrict__ tau32, int k,
              const unsigned* __restrict__ maxnorm_bits, int64_t* __restrict__ nbr, double* __restrict__ dist,
              int* __restrict__ flagged, int* __restrict__ nflag) {
  __shared__ double kd[8][kMaxKp];
  __shared__ int kc[8][kMaxKp];
  __shared__ double tk[8][kMaxKp];
  __shared__ int ts[8][kMaxKp];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t q = (int64_t)blockIdx.x * 8 + w;
  if (q >= n) return;
  const double* xq = X64 + q * DP;
  double qn = 0.0;  // centred norm of the query
  for (int t = 0; t < d; ++t) {
    const double c = xq[t] - mean[t];
    qn = fma(c, c, qn);
  }
  qn = sqrt(qn);
  for (int s = lane; s < kMaxKp; s += 32) {
    const int c = s < Kp ? cand[q * Kp + s] : -1;
    double dd = DBL_MAX;
    if (c >= 0) {
      const double* xc = X64 + (int64_t)c * DP;
      // sequential, unfused sum of squares: the reference's squared_euclidean
      dd = 0.0;
      for (int t = 0; t < d; ++t) {
        const double df = __dsub_rn(xq[t], xc[t]);
        dd = __dadd_rn(dd, __dmul_rn(df, df));
      }
    }
    kd[w][s] = dd;
    kc[w][s] = c >= 0 ? c : 0x7fffffff;
  }
  __syncwarp();
  warp_bitonic<double>(kd[w], kc[w], kMaxKp);
  // Certificate.  Every point j outside the list has FP32 distance
  // d32(j) >= tau32.  With u = 2^-24, N = |x_q - mean| + max_j |x_j - mean|
  // and D the exact squared distance, rounding the centred coordinates to FP32
  // and the FP32 fused sum of squares give
  //   |d32 - D| <= 4.1 u N sqrt(D) + (d+1) u D + 5 u^2 N^2,
  // so every outside point has D >= L, the positive root bound of
  //   (1 + (d+1)u) s^2 + 4.1 u N s - (tau32 - 5 u^2 N^2) >= 0,  D = s^2.
  // If L exceeds the k-th FP64 distance among the candidates, the FP64 top-k
  // is exact.
  const double u = 5.9604644775390625e-08;
  const double N = qn + (double)__uint_as_float(*maxnorm_bits);
  const double t32 = (double)tau32[q];
  const double qa = 1.0 + (double)(d + 1) * u, qb = 4.1 * u * N, qc = t32 - 5.0 * u * u * N * N;
  const double sroot = qc > 0.0 ? (-qb + sqrt(qb * qb + 4.0 * qa * qc)) / (2.0 * qa) : 0.0;
  const double lower = sroot * sroot * (1.0 - 4.0 * u);  // absorb the rounding of this bound itself
  const double dk = kd[w][k - 1];
  const bool full = kc[w][k - 1] != 0x7fffffff;
  const bool all_seen = t32 >= 3.0e38;  // fewer than Kp points: every point is a candidate
  const bool exact = full && (all_seen || lower > dk);
  if (!exact) {
    if (lane == 0) flagged[atomicAdd(nflag, 1)] = (int)q;
    return;
  }
  emit_row(q, k, kd[w], kc[w], tk[w], ts[w], nbr, dist);
}

// Rows of the queries that the certificate rejected, from the exact FP64 scan.
__global__ void __launch_bounds__(256)
finalize_kernel(const int* __restrict__ flagged, const int* __restrict__ nflag, const int* __restrict__ cand,
                const double* __restrict__ cand_d, int k, int64_t* __restrict__ nbr, double* __restrict__ dist) {
  __shared__ double kd[8][kMaxKp];
  __shared__ int kc[8][kMaxKp];
  __shared__ double tk[8][kMaxKp];
  __shared__ int ts[8][kMaxKp];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t slot = (int64_t)blockIdx.x * 8 + w;
  if (slot >= *nflag) return;
  const int64_t q = flagged[slot];
  for (int s = lane; s < k; s += 32) {
    kd[w][s] = cand_d[slot * k + s];
    kc[w][s] = cand[slot * k + s];
  }
  __syncwarp();
  emit_row(q, k, kd[w], kc[w], tk[w], ts[w], nbr, dist);
}

__global__ void zero_int(int* p, unsigned* u) {
  *p = 0;
  *u = 0u;
}

struct KnnScratch {
  double* mpart;
  double* mean;
  float* XT;
  float* nrm;
  unsigned char* TC;  // tensor-core operand tiles (DP == 32 only)
  double* X64;
  int* cand;
  float* tau32;
  int* flagged;
  int* fcand;
  double* fcand_d;
  int* nflag;
  unsigned* maxnorm;
  int64_t bytes;
};

constexpr int64_t align256(int64_t x) { return (x + 255) / 256 * 256; }

// Byte offsets of the scratch regions (each 256-byte aligned) and the total;
// constexpr so that the allocation-free entry point can size its fixed array
// from the same arithmetic.
struct KnnOffsets {
  int64_t mp, mean, XT, nrm, TC, X64, cand, tau, flagged, fcand, fcand_d, counters, bytes;
};

constexpr KnnOffsets knn_offsets(int64_t n, int DP, int k, int Kp) {
  KnnOffsets o{};
  int64_t at = 0;
  const int64_t npad = (n + kFC - 1) / kFC * kFC;
  o.mp = at; at += align256((int64_t)kMeanParts * 64 * 8);
  o.mean = at; at += align256(64 * 8);
  o.XT = at; at += align256(npad * DP * 4);
  o.nrm = at; at += align256(npad * 4);
  o.TC = at; at += DP == 32 ? align256(npad / kFC * kTTile) : 0;
  o.X64 = at; at += align256(n * DP * 8);
  o.cand = at; at += align256(n * (int64_t)Kp * 4);
  o.tau = at; at += align256(n * 4);
  o.flagged = at; at += align256(n * 4);
  o.fcand = at; at += align256(n * (int64_t)k * 4);
  o.fcand_d = at; at += align256(n * (int64_t)k * 8);
  o.counters = at; at += align256(16);
  o.bytes = at;
  return o;
}

KnnScratch knn_layout(char* base, int64_t n, int DP, int k, int Kp) {
  const KnnOffsets o = knn_offsets(n, DP, k, Kp);
  KnnScratch s{};
  if (base) {
    s.mpart = (double*)(base + o.mp);
    s.mean = (double*)(base + o.mean);
    s.XT = (float*)(base + o.XT);
    s.nrm = (float*)(base + o.nrm);
    s.TC = DP == 32 ? (unsigned char*)(base + o.TC) : nullptr;
    s.X64 = (double*)(base + o.X64);
    s.cand = (int*)(base + o.cand);
    s.tau32 = (float*)(base + o.tau);
    s.flagged = (int*)(base + o.flagged);
    s.fcand = (int*)(base + o.fcand);
    s.fcand_d = (double*)(base + o.fcand_d);
    s.nflag = (int*)(base + o.counters);
    s.maxnorm = (unsigned*)(base + o.counters + 8);
  }
  s.bytes = o.bytes;
  return s;
}

inline int pad_dim(int d) { return d <= 16 ? 16 : (d <= 32 ? 32 : 64); }

template <typename TD, int DP>
int launch_scan(const TD* Xp, int64_t n, const int* qlist, const int* qcount, int Kp, int* cand, TD* cand_d,
                TD* tau, cudaStream_t s) {
  const size_t smem = sizeof(ScanSmem<TD, DP>);
  if (cudaFuncSetAttribute(scan_kernel<TD, DP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  const int64_t grid = (n + kQT - 1) / kQT;
  scan_kernel<TD, DP><<<(unsigned)grid, kLW * 32, smem, s>>>(Xp, n, qlist, qcount, Kp, cand, cand_d, tau);
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

template <int DP, int LIST>
int launch_filter_scan_l(const float* XT, const float* nrm, int64_t n, int d, int Kp, int* cand, float* tau,
                         cudaStream_t s) {
  const size_t smem = sizeof(FilterSmem<DP, LIST>);
  if (cudaFuncSetAttribute(filter_scan_kernel<DP, LIST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  const int64_t grid = (n + kFQ - 1) / kFQ;
  filter_scan_kernel<DP, LIST><<<(unsigned)grid, kFW * 32, smem, s>>>(XT, nrm, n, d, Kp, cand, tau);
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

template <int DP>
int launch_filter_scan(const float* XT, const float* nrm, int64_t n, int d, int Kp, int* cand, float* tau,
                       cudaStream_t s) {
  if (Kp + 32 <= 128) return launch_filter_scan_l<DP, 128>(XT, nrm, n, d, Kp, cand, tau, s);
  return launch_filter_scan_l<DP, 256>(XT, nrm, n, d, Kp, cand, tau, s);
}

// The tensor-core filter serves up to 32 dimensions and lists of Kp + one
// chunk; SNAPGB300_KNN_FILTER=simt selects the FP32 filter (both give the
// same candidate lists).
bool use_tensor_filter(int DP, int Kp) {
  if (DP != 32 || Kp + kTChunk > kTList) return false;
  const char* e = getenv("SNAPGB300_KNN_FILTER");
  return !(e && strcmp(e, "simt") == 0);
}

int launch_tc_filter(const float* XT, const unsigned char* TC, const float* nrm, int64_t n, int d, int Kp, int* cand,
                     float* tau, cudaStream_t s) {
  const size_t smem = sizeof(TcSmem);
  if (cudaFuncSetAttribute(tc_filter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return SG_ERR_CUDA;
  const int64_t grid = (n + kTQ - 1) / kTQ;
  tc_filter_kernel<<<(unsigned)grid, kTThreads, smem, s>>>(XT, TC, nrm, n, d, Kp, cand, tau);
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

template <int DP>
int knn_run(const double* X, int64_t n, int d, int k, int Kp, const KnnScratch& w, int64_t* nbr, double* dist,
            cudaStream_t s) {
  zero_int<<<1, 1, 0, s>>>(w.nflag, w.maxnorm);
  mean_partial<<<kMeanParts, 64, 0, s>>>(X, n, d, w.mpart);
  mean_reduce<<<1, 64, 0, s>>>(w.mpart, kMeanParts, n, d, w.mean);
  prep_kernel<DP><<<grid_for(n, 256, 4096), 256, 0, s>>>(X, n, d, w.mean, w.XT, w.nrm, w.X64, w.maxnorm);
  SG_CHECK_LAUNCH();
  int e;
  if (use_tensor_filter(DP, Kp)) {
    tc_prep_kernel<<<grid_for(n, 256, 4096), 256, 0, s>>>(w.XT, w.nrm, n, w.TC);
    SG_CHECK_LAUNCH();
    e = launch_tc_filter(w.XT, w.TC, w.nrm, n, d, Kp, w.cand, w.tau32, s);
  } else {
    e = launch_filter_scan<DP>(w.XT, w.nrm, n, d, Kp, w.cand, w.tau32, s);
  }
  if (e) return e;
  rerank_kernel<DP><<<(unsigned)((n + 7) / 8), 256, 0, s>>>(w.X64, n, d, w.mean, w.cand, Kp, w.tau32, k,
                                                            w.maxnorm, nbr, dist, w.flagged, w.nflag);
  SG_CHECK_LAUNCH();
  // exact FP64 scan of the rejected queries (CTAs past the count exit at once)
  e = launch_scan<double, DP>(w.X64, n, w.flagged, w.nflag, k, w.fcand, w.fcand_d, nullptr, s);
  if (e) return e;
  finalize_kernel<<<(unsigned)((n + 7) / 8), 256, 0, s>>>(w.flagged, w.nflag, w.fcand, w.fcand_d, k, nbr, dist);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int64_t sg_knn_scratch_bytes(int64_t n, int d, int k, int margin) {
  if (n <= 0 || d <= 0 || d > 64 || k <= 0 || margin < 0) return -1;
  const int Kp = k + margin;
  return knn_layout(nullptr, n, pad_dim(d), k, Kp).bytes;
}

extern "C" int sg_knn(const double* X, int64_t n, int d, int k, int margin, int64_t* nbr, double* dist,
                      void* scratch, int64_t scratch_bytes, int* n_fallback, void* stream) {
  if (n < 2 || d <= 0 || d > 64 || k <= 0 || k > n - 1 || margin < 0 || n > 0x7fffffffLL) return SG_ERR_ARG;
  int Kp = k + margin;
  if (Kp > kMaxKp) Kp = kMaxKp;
  if (Kp > n - 1) Kp = (int)(n - 1);
  if (k > Kp) return SG_ERR_ARG;
  if (((uintptr_t)scratch & 255u) != 0) return SG_ERR_ARG;
  const int DP = pad_dim(d);
  KnnScratch w = knn_layout((char*)scratch, n, DP, k, k + margin);
  if (scratch_bytes < w.bytes) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  int e;
  if (DP == 16) e = knn_run<16>(X, n, d, k, Kp, w, nbr, dist, s);
  else if (DP == 32) e = knn_run<32>(X, n, d, k, Kp, w, nbr, dist, s);
  else e = knn_run<64>(X, n, d, k, Kp, w, nbr, dist, s);
  if (e) return e;
  if (n_fallback &&
      cudaMemcpyAsync(n_fallback, w.nflag, sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return SG_ERR_CUDA;
  return SG_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of sg_knn.
//
// Some callers cannot allocate device memory for the scratch sg_knn needs:
// an application whose device memory is owned by its own pool or framework
// (raw cudaMalloc is not allowed there), or a latency-bound caller for whom
// cudaMalloc, which may synchronise the whole device and is slow, is not an
// option.  For them the scratch lives in the fixed array below, which is part
// of this library's device image: every GPU that loads the library holds it
// (about 33 MB) until the process exits.
// ---------------------------------------------------------------------------
namespace sg {
namespace {

constexpr int64_t kNoAllocMaxN = 16384;  // points
constexpr int kNoAllocMaxDim = 32;       // dimensions
constexpr int kNoAllocMaxK = 100;        // neighbours
// sized by the scratch layout of the largest accepted problem: 16,384
// points (whole 128-point tiles), 32 dimensions (the tensor-core operand
// tiles are included), k = 100, candidate lists of kMaxKp
static_assert(kNoAllocMaxN % kFC == 0, "no-alloc capacity must be whole tiles");
constexpr int64_t kNoAllocBytes = knn_offsets(kNoAllocMaxN, kNoAllocMaxDim, kNoAllocMaxK, kMaxKp).bytes;

static __device__ __align__(256) unsigned char g_knn_scratch[kNoAllocBytes];

// Device address of g_knn_scratch on the current device.  In host code the
// name g_knn_scratch is only a host-side stand-in, so the address is looked
// up with the device current and the return code checked.  The lookup is
// repeated on every call (it is a table lookup in the CUDA runtime): a cached
// address would go stale when the device's context is destroyed and made
// again (cudaDeviceReset), which reloads the module at a new address.  The
// first lookup on a device loads the module that holds the array (CUDA's
// lazy module loading).
int knn_scratch_address(void** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_knn_scratch) != cudaSuccess || !p) return SG_ERR_CUDA;
  *out = p;
  return SG_OK;
}

}  // namespace
}  // namespace sg

extern "C" int sg_knn_noalloc(const double* X, int64_t n, int d, int k, int margin, int64_t* nbr, double* dist,
                              int* n_fallback, void* stream) {
  if (n < 2 || d <= 0 || k <= 0 || k > n - 1 || margin < 0) return SG_ERR_ARG;
  if (n > kNoAllocMaxN || d > kNoAllocMaxDim || k > kNoAllocMaxK) return SG_ERR_CAP;
  if (k + margin > kMaxKp) margin = kMaxKp - k;
  int Kp = k + margin;
  if (Kp > n - 1) Kp = (int)(n - 1);
  void* base = nullptr;
  int e = knn_scratch_address(&base);
  if (e) return e;
  const int DP = pad_dim(d);
  KnnScratch w = knn_layout((char*)base, n, DP, k, k + margin);
  if (w.bytes > kNoAllocBytes) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  // knn_run clears the two counters it accumulates into (fallback count,
  // max norm) before use; every other scratch byte is written before read.
  e = DP == 16 ? knn_run<16>(X, n, d, k, Kp, w, nbr, dist, s) : knn_run<32>(X, n, d, k, Kp, w, nbr, dist, s);
  if (e) return e;
  if (n_fallback &&
      cudaMemcpyAsync(n_fallback, w.nflag, sizeof(int), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return SG_ERR_CUDA;
  return SG_OK;
}
