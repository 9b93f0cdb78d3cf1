// Dense block kernels of the thick-restart block Lanczos (Krylov-Schur)
// eigensolver that replaces the reference's ARPACK call
// (snapatac2-python/src/embedding.rs:155-171, eigsh which='LM').
//
// Layout: the basis Q is n x ldq row-major (each cell's basis coefficients
// contiguous), the working block W is n x B row-major.  T = float (mixed
// precision) or double (all-FP64).  Every reduction across rows goes through
// per-CTA partials summed in a fixed order in FP64, so results are
// bit-reproducible run to run.
//
//   proj    C = Q[:, :ncols]ᵀ W           (ncols x B, FP64)
//   update  W -= Q[:, :ncols] C
//   cholqr  G = WᵀW, G = RᵀR (FP64 Cholesky), W <- W R⁻¹
//   finish  Q[:, col:col+B] = W, Z = W, Zs = a ⊙ W
//   hblock  Rayleigh-quotient diagonal block and coupling R into H (FP64)
//   rotate  out = Q[:, :m] Y                (thick restart, Ritz vectors)
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kProjBlock = 256;
constexpr int kProjRows = 32;

int sm_count_l() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// part[blk][p][c] = sum over this CTA's rows of Q[i,p] W[i,c]
template <typename T, int B, int CPT>
__global__ void __launch_bounds__(kProjBlock)
proj_partial(int64_t n, const T* __restrict__ Q, int64_t ldq, int ncols, const T* __restrict__ W,
             double* __restrict__ part) {
  __shared__ T ws[kProjRows][B];
  const int nb = gridDim.x, b = blockIdx.x;
  const int64_t r0 = n * b / nb, r1 = n * (b + 1) / nb;
  T acc[CPT][B];
#pragma unroll
  for (int q = 0; q < CPT; ++q)
#pragma unroll
    for (int c = 0; c < B; ++c) acc[q][c] = T(0);
  for (int64_t base = r0; base < r1; base += kProjRows) {
    const int nr = (r1 - base) < kProjRows ? (int)(r1 - base) : kProjRows;
    __syncthreads();
    for (int t = threadIdx.x; t < kProjRows * B; t += kProjBlock) {
      const int i = t / B, c = t % B;
      ws[i][c] = i < nr ? W[(base + i) * B + c] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const int p = threadIdx.x + q * kProjBlock;
      if (p < ncols) {
        // several rows' loads in flight, then their FMAs in row order
        constexpr int RU = sizeof(T) == 8 ? (B * CPT >= 8 ? 2 : 8) : (B * CPT >= 32 ? 4 : 8);
        for (int i0 = 0; i0 < nr; i0 += RU) {
          T qv[RU];
#pragma unroll
          for (int u = 0; u < RU; ++u) qv[u] = i0 + u < nr ? Q[(base + i0 + u) * ldq + p] : T(0);
#pragma unroll
          for (int u = 0; u < RU; ++u)
            if (i0 + u < nr) {
#pragma unroll
              for (int c = 0; c < B; ++c) acc[q][c] = fma(qv[u], ws[i0 + u][c], acc[q][c]);
            }
        }
      }
    }
  }
#pragma unroll
  for (int q = 0; q < CPT; ++q) {
    const int p = threadIdx.x + q * kProjBlock;
    if (p < ncols) {
#pragma unroll
      for (int c = 0; c < B; ++c) part[((int64_t)b * ncols + p) * B + c] = (double)acc[q][c];
    }
  }
}

// Gram partials of a block: part[blk][i*B + j] = sum over this CTA's rows of
// W[r,i] W[r,j].  Thread per row (all threads busy, unlike the projection
// kernel with only B basis columns); upper triangle in registers, then a
// fixed-order reduction over the CTA's threads (deterministic).
template <typename T, int B>
__global__ void __launch_bounds__(256) gram_partial(int64_t n, const T* __restrict__ W, double* __restrict__ part) {
  constexpr int NT = B * (B + 1) / 2;
  __shared__ double red[256 / 32][NT];
  const int nb = gridDim.x, b = blockIdx.x;
  const int64_t r0 = n * b / nb, r1 = n * (b + 1) / nb;
  T acc[NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) acc[t] = T(0);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += 256) {
    T w[B];
#pragma unroll
    for (int i = 0; i < B; ++i) w[i] = W[r * B + i];
    int t = 0;
#pragma unroll
    for (int i = 0; i < B; ++i)
#pragma unroll
      for (int j = i; j < B; ++j) {
        acc[t] = fma(w[i], w[j], acc[t]);
        ++t;
      }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    double v = (double)acc[t];
#pragma unroll
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][t] = v;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < NT; t += 256) {
    double v = 0.0;
    for (int w2 = 0; w2 < 256 / 32; ++w2) v += red[w2][t];
    // position t -> (i, j) of the packed upper triangle
    int i = 0, rem = t;
    while (rem >= B - i) { rem -= B - i; ++i; }
    const int j = i + rem;
    part[(int64_t)b * B * B + i * B + j] = v;
    part[(int64_t)b * B * B + j * B + i] = v;
  }
}

// C[t] = sum over the nparts partials of part[b][t], t < tot = ncols * B.  A
// CTA owns 32 consecutive outputs (lane = output, coalesced reads); warp w
// sums the partials b = w, w + 32, ... in order, then the 32 warp sums are
// added in warp order: a fixed order, so the result is deterministic.
constexpr int kReduceWarps = 32;
__global__ void __launch_bounds__(kReduceWarps * 32)
proj_reduce(int nparts, int ncols, int B, const double* __restrict__ part, double* __restrict__ C) {
  __shared__ double ws[kReduceWarps][33];
  const int tot = ncols * B;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int t = blockIdx.x * 32 + lane;
  double s = 0.0;
  if (t < tot) {
    int b = w;
    for (; b + 3 * kReduceWarps < nparts; b += 4 * kReduceWarps) {
      const double v0 = part[(int64_t)b * tot + t], v1 = part[(int64_t)(b + kReduceWarps) * tot + t];
      const double v2 = part[(int64_t)(b + 2 * kReduceWarps) * tot + t];
      const double v3 = part[(int64_t)(b + 3 * kReduceWarps) * tot + t];
      s += v0;
      s += v1;
      s += v2;
      s += v3;
    }
    for (; b < nparts; b += kReduceWarps) s += part[(int64_t)b * tot + t];
  }
  ws[w][lane] = s;
  __syncthreads();
  if (w == 0 && t < tot) {
    double r = 0.0;
    for (int k = 0; k < kReduceWarps; ++k) r += ws[k][lane];
    C[t] = r;
  }
}

// W[i,:] -= Q[i, :ncols] C   (one warp per row; lanes over basis columns).
// Each lane loads up to eight basis entries of the row before using them; the
// B column sums are then combined by a transpose butterfly (lane pairs swap
// half of their sums at each step), which leaves each column's full sum in
// the 32/B lanes whose high bits spell its index, with B - 1 + 5 - log2(B)
// shuffles instead of 5 B.  Fixed order: deterministic.
template <typename T, int B>
__global__ void __launch_bounds__(256)
update_kernel(int64_t n, const T* __restrict__ Q, int64_t ldq, int ncols, const double* __restrict__ C,
              T* __restrict__ W) {
  extern __shared__ __align__(16) unsigned char sraw[];
  T* cs = reinterpret_cast<T*>(sraw);  // ncols x B
  for (int t = threadIdx.x; t < ncols * B; t += blockDim.x) cs[t] = (T)C[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < n; i += nw) {
    T acc[B];
#pragma unroll
    for (int c = 0; c < B; ++c) acc[c] = T(0);
    for (int p0 = 0; p0 < ncols; p0 += 8 * 32) {
      T qv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int p = p0 + u * 32 + lane;
        qv[u] = p < ncols ? Q[i * ldq + p] : T(0);
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int p = p0 + u * 32 + lane;
        if (p < ncols) {
          // C's row p read as 16-byte vectors: word-wise reads at a B-word
          // stride put several lanes on one shared-memory bank; the FMAs
          // and their order are unchanged
          using VT = typename V16<T>::type;
          constexpr int VW = V16<T>::n;
          const VT* cv = reinterpret_cast<const VT*>(cs + (size_t)p * B);
#pragma unroll
          for (int j = 0; j < B / VW; ++j) {
            const VT c4 = cv[j];
            const T* cc = reinterpret_cast<const T*>(&c4);
#pragma unroll
            for (int q = 0; q < VW; ++q) acc[j * VW + q] = fma(qv[u], cc[q], acc[j * VW + q]);
          }
        }
      }
    }
    warp_colsum<T, B>(acc, lane);
    // the halvings used lane bits 16, 8, ... (B of the 32 lanes' patterns);
    // the upper half at each step adds half to the column index.  Lanes that
    // differ only in the remaining low bits hold the same sum; the one with
    // those bits zero writes it.
    int col = 0, live = B;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
      if (live > 1) {
        live /= 2;
        if (lane & o) col += live;
      }
    }
    if ((lane % (32 / B)) == 0) W[i * B + col] -= acc[0];
  }
}

// ---- FP32 tiled forms of proj and update -----------------------------------
// The basis is read in stages of 32 columns (128 bytes of a row; 16 in the
// update, whose smaller rings let three CTAs share an SM) by
// cp.async into per-warp shared-memory rings; rows of a staged tile are
// padded by 4 floats (36 or 20), so the 16-byte reads of eight consecutive
// rows touch 32 distinct banks.  Columns past ncols and rows past the limit are
// zero-filled by the copy itself (src-size < 16), so the inner loops have no
// bounds tests.  Only used when Q, W and every row start are 16-byte aligned.
constexpr int kStageCols = 32;
constexpr int kPitch = kStageCols + 4;
constexpr int kTileWarps = 4;

__device__ __forceinline__ void cp_async16(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// rows [row0, row0 + R) x columns [col0, col0 + SC) of Q into buf (R rows of
// SC + 4 floats); rows at or past rlim and columns at or past ncols read as
// zero.  Rows of SC + 4 floats (SC = 16 or 32) put the 16-byte reads of eight
// consecutive rows on 32 distinct banks.
template <int R, int SC = kStageCols>
__device__ __forceinline__ void stage_q(float* buf, const float* __restrict__ Q, int64_t ldq, int64_t rlim,
                                        int ncols, int64_t row0, int col0, int lane) {
  constexpr int CPR = SC / 4;  // 16-byte chunks per row
#pragma unroll
  for (int j = 0; j < R * CPR / 32; ++j) {
    const int idx = j * 32 + lane;
    const int r = idx / CPR, c = (idx % CPR) * 4;
    const int64_t row = row0 + r;
    const int col = col0 + c;
    int bytes = (ncols - col) * 4;
    bytes = bytes < 0 ? 0 : (bytes > 16 ? 16 : bytes);
    if (row >= rlim) bytes = 0;
    cp_async16(buf + r * (SC + 4) + c, bytes ? Q + row * ldq + col : Q, bytes);
  }
}

// basis columns per stage of the update: 16 (smaller rings, three CTAs per SM)
constexpr int kUpdCols = 16;
constexpr int kUpdPitch = kUpdCols + 4;

// W -= Q[:, :ncols] C.  Each warp owns 64-row tiles (rows lane and lane + 32
// of a tile per lane, all B columns in registers); C (FP32, zero past ncols)
// sits in shared memory and is read as broadcasts.  The warp walks (tile,
// stage) in order with a two-deep cp.async ring.  Each row's sum runs over
// the columns in ascending order: deterministic.
template <int B>
__global__ void __launch_bounds__(kTileWarps * 32)
update_tiled(int64_t n, const float* __restrict__ Q, int64_t ldq, int ncols, const double* __restrict__ C,
             float* __restrict__ W) {
  constexpr int R = 64;
  extern __shared__ __align__(16) unsigned char sraw[];
  const int nch = (ncols + kUpdCols - 1) / kUpdCols;
  float* cs = reinterpret_cast<float*>(sraw);
  float* ring = cs + (size_t)nch * kUpdCols * B;
  for (int t = threadIdx.x; t < nch * kUpdCols * B; t += blockDim.x) cs[t] = t < ncols * B ? (float)C[t] : 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float* buf = ring + (size_t)wid * 2 * R * kUpdPitch;
  const int64_t ntiles = (n + R - 1) / R;
  const int64_t nw = (int64_t)gridDim.x * kTileWarps;
  int64_t tile = blockIdx.x * (int64_t)kTileWarps + wid;
  if (tile >= ntiles) return;
  int ch = 0, sl = 0;
  stage_q<R, kUpdCols>(buf, Q, ldq, n, ncols, tile * R, 0, lane);
  cp_async_commit();
  float a0[B], a1[B];
#pragma unroll
  for (int c = 0; c < B; ++c) a0[c] = a1[c] = 0.f;
  while (true) {
    int64_t ntile = tile;
    int nchk = ch + 1;
    if (nchk == nch) {
      nchk = 0;
      ntile = tile + nw;
    }
    const bool more = ntile < ntiles;
    if (more) stage_q<R, kUpdCols>(buf + (sl ^ 1) * R * kUpdPitch, Q, ldq, n, ncols, ntile * R, nchk * kUpdCols, lane);
    cp_async_commit();
    cp_async_wait<1>();
    __syncwarp();
    const float* qb = buf + sl * R * kUpdPitch;
    const float* cst = cs + (size_t)ch * kUpdCols * B;
#pragma unroll 2
    for (int p4 = 0; p4 < kUpdCols / 4; ++p4) {
      const float4 qa = *reinterpret_cast<const float4*>(qb + lane * kUpdPitch + 4 * p4);
      const float4 qc = *reinterpret_cast<const float4*>(qb + (lane + 32) * kUpdPitch + 4 * p4);
      const float va[4] = {qa.x, qa.y, qa.z, qa.w}, vc[4] = {qc.x, qc.y, qc.z, qc.w};
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4* cv = reinterpret_cast<const float4*>(cst + (4 * p4 + q) * B);
#pragma unroll
        for (int j = 0; j < B / 4; ++j) {
          const float4 c4 = cv[j];
          a0[4 * j + 0] = fmaf(va[q], c4.x, a0[4 * j + 0]);
          a0[4 * j + 1] = fmaf(va[q], c4.y, a0[4 * j + 1]);
          a0[4 * j + 2] = fmaf(va[q], c4.z, a0[4 * j + 2]);
          a0[4 * j + 3] = fmaf(va[q], c4.w, a0[4 * j + 3]);
          a1[4 * j + 0] = fmaf(vc[q], c4.x, a1[4 * j + 0]);
          a1[4 * j + 1] = fmaf(vc[q], c4.y, a1[4 * j + 1]);
          a1[4 * j + 2] = fmaf(vc[q], c4.z, a1[4 * j + 2]);
          a1[4 * j + 3] = fmaf(vc[q], c4.w, a1[4 * j + 3]);
        }
      }
    }
    __syncwarp();
    if (ch == nch - 1) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t row = tile * R + lane + 32 * h;
        if (row < n) {
          float4* wr = reinterpret_cast<float4*>(W + row * B);
#pragma unroll
          for (int j = 0; j < B / 4; ++j) {
            float4 v = wr[j];
            const float* a = h ? a1 : a0;
            v.x -= a[4 * j + 0];
            v.y -= a[4 * j + 1];
            v.z -= a[4 * j + 2];
            v.w -= a[4 * j + 3];
            wr[j] = v;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < B; ++c) a0[c] = a1[c] = 0.f;
    }
    if (!more) break;
    tile = ntile;
    ch = nchk;
    sl ^= 1;
  }
  cp_async_wait<0>();
}

// part[blk][p][c] = sum over the CTA's rows [r0, r1) of Q[i,p] W[i,c].  Per
// stage of 32 columns the warps take the CTA's 32-row tiles in turn; a lane
// owns 4 columns p x B/4 columns c (lane = 8 column groups x 4 output
// groups), so per row it reads one 16-byte vector of Q and B/4 values of W.
// The four warps' FP32 sums are added in FP64 in warp order: deterministic.
template <int B>
__host__ __device__ constexpr int proj_stages() {
  return B >= 32 ? 2 : 3;
}

template <int B>
__global__ void __launch_bounds__(kTileWarps * 32)
proj_tiled(int64_t n, const float* __restrict__ Q, int64_t ldq, int ncols, const float* __restrict__ W,
           double* __restrict__ part) {
  constexpr int R = 32, CW = B / 4, kProjStages = proj_stages<B>();
  extern __shared__ __align__(16) unsigned char sraw[];
  double* red = reinterpret_cast<double*>(sraw);                           // [warps][32 * B]
  float* qring = reinterpret_cast<float*>(red + kTileWarps * kStageCols * B);  // [warps][stages][R][kPitch]
  float* wring = qring + kTileWarps * kProjStages * R * kPitch;            // [warps][stages][R][B]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int pg = lane >> 2, cg = lane & 3;
  const int nb = gridDim.x, b = blockIdx.x;
  const int64_t r0 = n * b / nb, r1 = n * (b + 1) / nb;
  const int ntc = (int)((r1 - r0 + R - 1) / R);
  const int ntw = ntc > wid ? (ntc - wid + kTileWarps - 1) / kTileWarps : 0;
  const int nch = (ncols + kStageCols - 1) / kStageCols;
  const int total = ntw * nch;
  float* qb = qring + (size_t)wid * kProjStages * R * kPitch;
  float* wb = wring + (size_t)wid * kProjStages * R * B;
  auto stage = [&](int i) {
    const int ch = i / ntw, j = i % ntw;
    const int64_t row0 = r0 + (int64_t)(wid + kTileWarps * j) * R;
    const int sl = i % kProjStages;
    stage_q<R>(qb + sl * R * kPitch, Q, ldq, r1, ncols, row0, ch * kStageCols, lane);
#pragma unroll
    for (int t = lane; t < R * CW; t += 32) {
      const int r = t / CW, c = (t % CW) * 4;
      const int64_t row = row0 + r;
      const int bytes = row < r1 ? 16 : 0;
      cp_async16(wb + (sl * R + r) * B + c, bytes ? W + row * B + c : W, bytes);
    }
  };
#pragma unroll
  for (int i = 0; i < kProjStages - 1; ++i) {
    if (i < total) stage(i);
    cp_async_commit();
  }
  int i = 0;
  for (int ch = 0; ch < nch; ++ch) {
    float acc[4][CW];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int c = 0; c < CW; ++c) acc[u][c] = 0.f;
    for (int j = 0; j < ntw; ++j, ++i) {
      if (i + kProjStages - 1 < total) stage(i + kProjStages - 1);
      cp_async_commit();
      cp_async_wait<kProjStages - 1>();
      __syncwarp();
      const int sl = i % kProjStages;
      const float* qs = qb + sl * R * kPitch + pg * 4;
      const float* ws = wb + sl * R * B + cg * CW;
#pragma unroll 4
      for (int r = 0; r < R; ++r) {
        const float4 q4 = *reinterpret_cast<const float4*>(qs + r * kPitch);
        const float qv[4] = {q4.x, q4.y, q4.z, q4.w};
        float wv[CW];
        if constexpr (CW % 4 == 0) {
#pragma unroll
          for (int c = 0; c < CW; c += 4) {
            const float4 w4 = *reinterpret_cast<const float4*>(ws + r * B + c);
            wv[c] = w4.x;
            wv[c + 1] = w4.y;
            wv[c + 2] = w4.z;
            wv[c + 3] = w4.w;
          }
        } else if constexpr (CW == 2) {
          const float2 w2 = *reinterpret_cast<const float2*>(ws + r * B);
          wv[0] = w2.x;
          wv[1] = w2.y;
        } else {
          wv[0] = ws[r * B];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int c = 0; c < CW; ++c) acc[u][c] = fmaf(qv[u], wv[c], acc[u][c]);
      }
      __syncwarp();
    }
    double* rw = red + (size_t)wid * kStageCols * B;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int c = 0; c < CW; ++c) rw[(pg * 4 + u) * B + cg * CW + c] = (double)acc[u][c];
    __syncthreads();
    for (int t = threadIdx.x; t < kStageCols * B; t += blockDim.x) {
      const int p = ch * kStageCols + t / B;
      if (p < ncols) {
        double s = red[t];
#pragma unroll
        for (int w2 = 1; w2 < kTileWarps; ++w2) s += red[(size_t)w2 * kStageCols * B + t];
        part[((int64_t)b * ncols + p) * B + t % B] = s;
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
}

size_t update_tiled_smem(int B, int ncols) {
  const int nch = (ncols + kUpdCols - 1) / kUpdCols;
  return (size_t)nch * kUpdCols * B * 4 + (size_t)kTileWarps * 2 * 64 * kUpdPitch * 4;
}

template <int B>
size_t proj_tiled_smem() {
  return (size_t)kTileWarps * kStageCols * B * 8 + (size_t)kTileWarps * proj_stages<B>() * 32 * (kPitch + B) * 4;
}

bool tiled_ok(const void* Q, int64_t ldq, const void* W) {
  return ((uintptr_t)Q & 15u) == 0 && ((uintptr_t)W & 15u) == 0 && (ldq & 3) == 0;
}

// Cholesky of the B x B Gram matrix (one warp, lane j owns column j):
// G = RᵀR with R upper triangular; also Rinv = R⁻¹.  A non-positive pivot
// relative to the diagonal sets SG_ERR_NUMERIC (rank-deficient block).  G is
// staged in shared memory first; lane j's column of R⁻¹ is built in shared
// memory (no per-thread local arrays).
__global__ void chol_kernel(int B, const double* __restrict__ G, double* __restrict__ R,
                            double* __restrict__ Rinv, int* status) {
  // FP64 divisions and square roots are long dependent chains on GB300's
  // FP64 unit: each pivot takes one reciprocal square root (r_kk = s·rsqrt(s),
  // 1/r_kk = rsqrt(s)) and every division becomes a product with it
  __shared__ double g[32][33];
  __shared__ double r[32][33];
  __shared__ double x[32][33];  // x[i][j]: row i of column j of R⁻¹
  __shared__ double rd[32];     // 1 / r[k][k]
  const int j = threadIdx.x;
  for (int t = j; t < B * B; t += 32) g[t / B][t % B] = G[t];
  for (int i = 0; i < B; ++i) {
    r[i][j] = 0.0;
    x[i][j] = 0.0;
  }
  __syncwarp();
  bool fail = false;
  for (int k = 0; k < B; ++k) {
    if (j == k) {
      double s = g[k][k];
      for (int i = 0; i < k; ++i) s -= r[i][k] * r[i][k];
      const double gkk = g[k][k];
      if (!(s > 1e-28 * (gkk > 0 ? gkk : 1.0)) || !(s > 0.0)) { fail = true; s = 1.0; }
      const double rs = rsqrt(s);
      r[k][k] = s * rs;
      rd[k] = rs;
    }
    __syncwarp();
    const double ip = rd[k];
    if (j > k && j < B) {
      double s = g[k][j];
      for (int i = 0; i < k; ++i) s -= r[i][k] * r[i][j];
      r[k][j] = s * ip;
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, fail) && j == 0) atomicCAS(status, 0, SG_ERR_NUMERIC);
  // back substitution, lane j computes column j of R^-1
  if (j < B) {
    x[j][j] = rd[j];
    for (int i = j - 1; i >= 0; --i) {
      double s = 0.0;
      for (int t = i + 1; t <= j; ++t) s += r[i][t] * x[t][j];
      x[i][j] = -s * rd[i];
    }
    for (int i = 0; i < B; ++i) {
      Rinv[i * B + j] = i <= j ? x[i][j] : 0.0;
      R[i * B + j] = r[i][j];
    }
  }
}

// W[i,:] <- W[i,:] Rinv, FP32 blocks of 16: thread per row, the row in
// registers, Rinv in shared memory read as broadcasts; column c sums
// W[i,k] Rinv[k,c] over k = 0..c in order (the order of the warp form)
template <int B>
__global__ void __launch_bounds__(256) apply_rinv_rows(int64_t n, const double* __restrict__ Rinv,
                                                      float* __restrict__ W) {
  __shared__ float ri[B][B];
  for (int t = threadIdx.x; t < B * B; t += blockDim.x) ri[t / B][t % B] = (float)Rinv[t];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    float w[B];
    const float4* wr = reinterpret_cast<const float4*>(W + i * B);
#pragma unroll
    for (int q = 0; q < B / 4; ++q) {
      const float4 v = wr[q];
      w[4 * q] = v.x;
      w[4 * q + 1] = v.y;
      w[4 * q + 2] = v.z;
      w[4 * q + 3] = v.w;
    }
    float4* wo = reinterpret_cast<float4*>(W + i * B);
#pragma unroll
    for (int q = 0; q < B / 4; ++q) {  // four output columns at a time
      float o[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int c = 4 * q + u;
        float s = 0.f;
#pragma unroll
        for (int k = 0; k <= c; ++k) s = fmaf(w[k], ri[k][c], s);
        o[u] = s;
      }
      wo[q] = make_float4(o[0], o[1], o[2], o[3]);
    }
  }
}

// W[i,:] <- W[i,:] Rinv for blocks of 16 or 32 (warp per row, lane c
// computes column c: W[i,k] Rinv[k,c] over k = 0..c in order)
template <typename T, int B>
__global__ void __launch_bounds__(256) apply_rinv_warp(int64_t n, const double* __restrict__ Rinv, T* __restrict__ W) {
  __shared__ T ri[B][B];
  for (int t = threadIdx.x; t < B * B; t += blockDim.x) ri[t / B][t % B] = (T)Rinv[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < n; i += nw) {
    const T w = lane < B ? W[i * B + lane] : T(0);
    T s = T(0);
#pragma unroll
    for (int k = 0; k < B; ++k) {
      const T wk = __shfl_sync(0xffffffffu, w, k);
      if (lane < B && k <= lane) s = fma(wk, ri[k][lane < B ? lane : 0], s);
    }
    if (lane < B) W[i * B + lane] = s;
  }
}

// W[i,:] <- W[i,:] Rinv for blocks of 4 or 8 (thread per row, same order)
template <typename T, int B>
__global__ void __launch_bounds__(256) apply_rinv(int64_t n, const double* __restrict__ Rinv, T* __restrict__ W) {
  __shared__ T ri[B][B];
  for (int t = threadIdx.x; t < B * B; t += blockDim.x) ri[t / B][t % B] = (T)Rinv[t];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T w[B], o[B];
#pragma unroll
    for (int k = 0; k < B; ++k) w[k] = W[i * B + k];
#pragma unroll
    for (int c = 0; c < B; ++c) {
      T s = T(0);
#pragma unroll
      for (int k = 0; k <= c; ++k) s = fma(w[k], ri[k][c], s);
      o[c] = s;
    }
#pragma unroll
    for (int c = 0; c < B; ++c) W[i * B + c] = o[c];
  }
}

// Q[i, col:col+B] = W[i,:]; Z = W (optional); Zs = a ⊙ W
template <typename T>
__global__ void finish_kernel(int64_t n, int B, const T* __restrict__ W, T* __restrict__ Q, int64_t ldq,
                              int col, T* __restrict__ Z, T* __restrict__ Zs, const T* __restrict__ a) {
  const int64_t tot = n * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / B;
    const int c = (int)(t % B);
    const T v = W[t];
    if (Q) Q[i * ldq + col + c] = v;
    if (Z) Z[t] = v;
    if (Zs) Zs[t] = a[i] * v;
  }
}

// H[m0:m0+B, m0:m0+B] = sym(C1 + C2 rows m0..m0+B); coupling R = R2 R1 into
// H[m0+B:m0+2B, m0:m0+B] and its transpose.
__global__ void hblock_kernel(int B, double* __restrict__ H, int64_t ldh, int m0, const double* __restrict__ C1,
                              const double* __restrict__ C2, const double* __restrict__ R1,
                              const double* __restrict__ R2, double* __restrict__ Rout, int write_coupling) {
  const int r = threadIdx.y, c = threadIdx.x;
  if (r >= B || c >= B) return;
  const double d1 = C1[(int64_t)(m0 + r) * B + c] + (C2 ? C2[(int64_t)(m0 + r) * B + c] : 0.0);
  const double d2 = C1[(int64_t)(m0 + c) * B + r] + (C2 ? C2[(int64_t)(m0 + c) * B + r] : 0.0);
  H[(int64_t)(m0 + r) * ldh + m0 + c] = 0.5 * (d1 + d2);
  // R = R2 R1 (both upper triangular)
  double s = 0.0;
  for (int k = 0; k < B; ++k) s += R2[r * B + k] * R1[k * B + c];
  if (Rout) Rout[r * B + c] = s;
  if (write_coupling) {
    H[(int64_t)(m0 + B + r) * ldh + m0 + c] = s;
    H[(int64_t)(m0 + c) * ldh + m0 + B + r] = s;
  }
}

// out[i, 0:k] = Q[i, 0:m] Y[0:m, 0:k]   (warp per row, lane = output column
// inside a 32-column tile given by blockIdx.y)
template <typename TQ, typename TA, typename TO>
__global__ void __launch_bounds__(256)
rotate_kernel(int64_t n, const TQ* __restrict__ Q, int64_t ldq, int m, const double* __restrict__ Y,
              int64_t ldy, int k, TO* __restrict__ out, int64_t ldo) {
  extern __shared__ __align__(16) unsigned char sraw[];
  TA* ys = reinterpret_cast<TA*>(sraw);  // m x 32
  const int q0 = blockIdx.y * 32;
  for (int t = threadIdx.x; t < m * 32; t += blockDim.x) {
    const int p = t / 32, q = t % 32;
    ys[t] = (q0 + q < k) ? (TA)Y[(int64_t)p * ldy + q0 + q] : TA(0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < n; i += nw) {
    TA acc = TA(0);
    for (int p0 = 0; p0 < m; p0 += 32) {
      const TA qv = (p0 + lane < m) ? (TA)Q[i * ldq + p0 + lane] : TA(0);
      const int lim = min(32, m - p0);
      for (int t = 0; t < lim; ++t) acc = fma(__shfl_sync(0xffffffffu, qv, t), ys[(p0 + t) * 32 + lane], acc);
    }
    if (q0 + lane < k) out[i * ldo + q0 + lane] = (TO)acc;
  }
}

// Uniform [-0.5, 0.5) values from a splitmix64 hash of (seed, index):
// deterministic and identical on every platform.
__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

template <typename T>
__global__ void fill_random(int64_t count, uint64_t seed, T* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < count; t += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t h = splitmix64(seed * 0x2545f4914f6cdd1dull + (uint64_t)t);
    out[t] = (T)((double)(h >> 11) * (1.0 / 9007199254740992.0) - 0.5);
  }
}

// largest dynamic shared memory of the tiled kernels (ncols <= 640, B = 32),
// the fixed cap set on them
constexpr int kTiledSmemCap = 200 * 1024;

template <int B>
int proj_tiled_launch(int64_t n, const float* Q, int64_t ldq, int ncols, const float* W, double* part, int nparts,
                      double* C, cudaStream_t s) {
  const size_t smem = proj_tiled_smem<B>();
  // set on every call (the attribute is per device); always the same fixed
  // cap, so concurrent callers cannot lower it under one another
  if (cudaFuncSetAttribute(proj_tiled<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTiledSmemCap) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  proj_tiled<B><<<nparts, kTileWarps * 32, smem, s>>>(n, Q, ldq, ncols, W, part);
  SG_CHECK_LAUNCH();
  proj_reduce<<<(ncols * B + 31) / 32, kReduceWarps * 32, 0, s>>>(nparts, ncols, B, part, C);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <typename T, int B>
int proj_t(int64_t n, const T* Q, int64_t ldq, int ncols, const T* W, double* part, int nparts, double* C,
           cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (tiled_ok(Q, ldq, W)) return proj_tiled_launch<B>(n, Q, ldq, ncols, W, part, nparts, C, s);
  }
  // column slices of at most 2 * kProjBlock basis vectors per launch (one
  // slice per thread column when a row of W is 128 bytes or more: two would
  // not fit the register file)
  constexpr int kSlice = (B * (int)sizeof(T) >= 128 ? 1 : 2) * kProjBlock;
  for (int c0 = 0; c0 < ncols; c0 += kSlice) {
    const int nc = ncols - c0 < kSlice ? ncols - c0 : kSlice;
    if constexpr (kSlice > kProjBlock) {
      if (nc > kProjBlock) proj_partial<T, B, 2><<<nparts, kProjBlock, 0, s>>>(n, Q + c0, ldq, nc, W, part);
      else proj_partial<T, B, 1><<<nparts, kProjBlock, 0, s>>>(n, Q + c0, ldq, nc, W, part);
    } else {
      proj_partial<T, B, 1><<<nparts, kProjBlock, 0, s>>>(n, Q + c0, ldq, nc, W, part);
    }
    SG_CHECK_LAUNCH();
    const int tot = nc * B;
    proj_reduce<<<(tot + 31) / 32, kReduceWarps * 32, 0, s>>>(nparts, nc, B, part, C + (int64_t)c0 * B);
    SG_CHECK_LAUNCH();
  }
  return SG_OK;
}

template <typename T>
int proj_dispatch(int B, int64_t n, const T* Q, int64_t ldq, int ncols, const T* W, double* part, int nparts,
                  double* C, cudaStream_t s) {
  switch (B) {
    case 4: return proj_t<T, 4>(n, Q, ldq, ncols, W, part, nparts, C, s);
    case 8: return proj_t<T, 8>(n, Q, ldq, ncols, W, part, nparts, C, s);
    case 16: return proj_t<T, 16>(n, Q, ldq, ncols, W, part, nparts, C, s);
    case 32: return proj_t<T, 32>(n, Q, ldq, ncols, W, part, nparts, C, s);
    default: return SG_ERR_ARG;
  }
}

template <int B>
int update_tiled_launch(int64_t n, const float* Q, int64_t ldq, int ncols, const double* C, float* W,
                        cudaStream_t s) {
  const size_t smem = update_tiled_smem(B, ncols);
  if (smem > (size_t)kTiledSmemCap) return SG_ERR_ARG;
  if (cudaFuncSetAttribute(update_tiled<B>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTiledSmemCap) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  int occ = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, update_tiled<B>, kTileWarps * 32, smem) != cudaSuccess)
    return SG_ERR_CUDA;
  const int per_sm = occ > 0 ? occ : 1;
  const int64_t tiles = (n + 63) / 64;
  const int64_t want = (tiles + kTileWarps - 1) / kTileWarps;
  const int64_t cap = (int64_t)per_sm * sm_count_l();
  const int grid = (int)(want < cap ? want : cap);
  update_tiled<B><<<grid, kTileWarps * 32, smem, s>>>(n, Q, ldq, ncols, C, W);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <typename T>
int update_dispatch(int B, int64_t n, const T* Q, int64_t ldq, int ncols, const double* C, T* W, cudaStream_t s) {
  if constexpr (sizeof(T) == 4) {
    if (tiled_ok(Q, ldq, W)) {
      switch (B) {
        case 4: return update_tiled_launch<4>(n, Q, ldq, ncols, C, W, s);
        case 8: return update_tiled_launch<8>(n, Q, ldq, ncols, C, W, s);
        case 16: return update_tiled_launch<16>(n, Q, ldq, ncols, C, W, s);
        case 32: return update_tiled_launch<32>(n, Q, ldq, ncols, C, W, s);
        default: return SG_ERR_ARG;
      }
    }
  }
  const int grid = grid_for(n * 32, 256, 8 * sm_count_l());
  const size_t smem = (size_t)ncols * B * sizeof(T);
  if (smem > 200 * 1024) return SG_ERR_ARG;
  // dynamic shared memory caps are set to the largest size (200 KB) any call
  // needs, never to one call's size: host threads embedding datasets of
  // different sizes concurrently would otherwise lower the cap between
  // another thread's set and its launch
#define SG_UPD(BB)                                                                                   \
  case BB:                                                                                           \
    if (smem > 48 * 1024 &&                                                                          \
        cudaFuncSetAttribute(update_kernel<T, BB>, cudaFuncAttributeMaxDynamicSharedMemorySize,      \
                             200 * 1024) != cudaSuccess)                                             \
      return SG_ERR_CUDA;                                                                            \
    update_kernel<T, BB><<<grid, 256, smem, s>>>(n, Q, ldq, ncols, C, W);                            \
    break;
  switch (B) {
    SG_UPD(4) SG_UPD(8) SG_UPD(16) SG_UPD(32)
    default: return SG_ERR_ARG;
  }
#undef SG_UPD
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <typename T>
int rinv_dispatch(int B, int64_t n, const double* Rinv, T* W, cudaStream_t s) {
  const int grid = grid_for(n, 256, 16 * sm_count_l());
  const int gridw = grid_for(n * 32, 256, 8 * sm_count_l());
  const bool rows_ok = sizeof(T) == 4 && ((uintptr_t)W & 15u) == 0;
  switch (B) {
    case 4: apply_rinv<T, 4><<<grid, 256, 0, s>>>(n, Rinv, W); break;
    case 8: apply_rinv<T, 8><<<grid, 256, 0, s>>>(n, Rinv, W); break;
    case 16:
      if (rows_ok) apply_rinv_rows<16><<<grid, 256, 0, s>>>(n, Rinv, reinterpret_cast<float*>(W));
      else apply_rinv_warp<T, 16><<<gridw, 256, 0, s>>>(n, Rinv, W);
      break;
    case 32: apply_rinv_warp<T, 32><<<gridw, 256, 0, s>>>(n, Rinv, W); break;
    default: return SG_ERR_ARG;
  }
  SG_CHECK_LAUNCH();
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_proj_parts(void) { return 2 * sm_count_l(); }

extern "C" int sg_fill_random(int dtype, int64_t count, uint64_t seed, void* out, void* stream) {
  if (count < 0) return SG_ERR_ARG;
  if (count == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  const int grid = grid_for(count, 256, 16 * sm_count_l());
  if (dtype == 0) fill_random<float><<<grid, 256, 0, s>>>(count, seed, (float*)out);
  else if (dtype == 1) fill_random<double><<<grid, 256, 0, s>>>(count, seed, (double*)out);
  else return SG_ERR_ARG;
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_block_proj(int dtype, int block, int64_t n, const void* Q, int64_t ldq, int ncols,
                             const void* W, double* part, int nparts, double* C, void* stream) {
  if (n <= 0 || ncols <= 0 || nparts <= 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (dtype == 0) return proj_dispatch<float>(block, n, (const float*)Q, ldq, ncols, (const float*)W, part, nparts, C, s);
  if (dtype == 1) return proj_dispatch<double>(block, n, (const double*)Q, ldq, ncols, (const double*)W, part, nparts, C, s);
  return SG_ERR_ARG;
}

extern "C" int sg_block_update(int dtype, int block, int64_t n, const void* Q, int64_t ldq, int ncols,
                               const double* C, void* W, void* stream) {
  if (n <= 0 || ncols <= 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (dtype == 0) return update_dispatch<float>(block, n, (const float*)Q, ldq, ncols, C, (float*)W, s);
  if (dtype == 1) return update_dispatch<double>(block, n, (const double*)Q, ldq, ncols, C, (double*)W, s);
  return SG_ERR_ARG;
}

// One Cholesky-QR pass: G = WᵀW, G = RᵀR, W <- W R⁻¹.  G, R, Rinv: B x B FP64.
extern "C" int sg_block_cholqr(int dtype, int block, int64_t n, void* W, double* part, int nparts, double* G,
                               double* R, double* Rinv, int* status, void* stream) {
  if (n <= 0 || block < 1 || block > 32) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  int e = SG_OK;
  if (dtype == 0 && block == 8) gram_partial<float, 8><<<nparts, 256, 0, s>>>(n, (const float*)W, part);
  else if (dtype == 0 && block == 4) gram_partial<float, 4><<<nparts, 256, 0, s>>>(n, (const float*)W, part);
  else if (dtype == 1 && block == 8) gram_partial<double, 8><<<nparts, 256, 0, s>>>(n, (const double*)W, part);
  else if (dtype == 1 && block == 4) gram_partial<double, 4><<<nparts, 256, 0, s>>>(n, (const double*)W, part);
  else e = sg_block_proj(dtype, block, n, W, block, block, W, part, nparts, G, stream);
  if (e) return e;
  if (block == 4 || block == 8) {
    SG_CHECK_LAUNCH();
    proj_reduce<<<(block * block + 31) / 32, kReduceWarps * 32, 0, s>>>(nparts, block, block, part, G);
    SG_CHECK_LAUNCH();
  }
  chol_kernel<<<1, 32, 0, s>>>(block, G, R, Rinv, status);
  SG_CHECK_LAUNCH();
  if (dtype == 0) return rinv_dispatch<float>(block, n, Rinv, (float*)W, s);
  if (dtype == 1) return rinv_dispatch<double>(block, n, Rinv, (double*)W, s);
  return SG_ERR_ARG;
}

extern "C" int sg_block_finish(int dtype, int block, int64_t n, const void* W, void* Q, int64_t ldq, int col,
                               void* Z, void* Zs, const void* rowscale, void* stream) {
  if (n <= 0 || (Zs && !rowscale)) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int grid = grid_for(n * block, 256, 16 * sm_count_l());
  if (dtype == 0)
    finish_kernel<float><<<grid, 256, 0, s>>>(n, block, (const float*)W, (float*)Q, ldq, col, (float*)Z,
                                              (float*)Zs, (const float*)rowscale);
  else if (dtype == 1)
    finish_kernel<double><<<grid, 256, 0, s>>>(n, block, (const double*)W, (double*)Q, ldq, col, (double*)Z,
                                               (double*)Zs, (const double*)rowscale);
  else
    return SG_ERR_ARG;
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_lanczos_hblock(int block, double* H, int64_t ldh, int m0, const double* C1, const double* C2,
                                 const double* R1, const double* R2, double* Rout, int write_coupling,
                                 void* stream) {
  if (block < 1 || block > 32 || m0 < 0) return SG_ERR_ARG;
  hblock_kernel<<<1, dim3(block, block), 0, as_stream(stream)>>>(block, H, ldh, m0, C1, C2, R1, R2, Rout,
                                                                 write_coupling);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// out[:, 0:k] = Q[:, 0:m] Y[0:m, 0:k].  tq/to: 0 = float, 1 = double (the
// accumulation runs in the wider of the two).
extern "C" int sg_basis_rotate(int tq, int to, int64_t n, const void* Q, int64_t ldq, int m, const double* Y,
                               int64_t ldy, int k, void* out, int64_t ldo, void* stream) {
  if (n <= 0 || m <= 0 || k <= 0 || m > 1536) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int gx = grid_for(n * 32, 256, 8 * sm_count_l());
  dim3 grid(gx, (k + 31) / 32);
  const bool wide = tq == 1 || to == 1;
  const size_t smem = (size_t)m * 32 * (wide ? sizeof(double) : sizeof(float));
  if (smem > 200 * 1024) return SG_ERR_ARG;
#define SG_ROT(TQ, TA, TO)                                                                              \
  do {                                                                                                  \
    if (smem > 48 * 1024 &&                                                                             \
        cudaFuncSetAttribute(rotate_kernel<TQ, TA, TO>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                             200 * 1024) != cudaSuccess)                                                \
      return SG_ERR_CUDA;                                                                               \
    rotate_kernel<TQ, TA, TO><<<grid, 256, smem, s>>>(n, (const TQ*)Q, ldq, m, Y, ldy, k, (TO*)out, ldo); \
  } while (0)
  if (tq == 0 && to == 0) SG_ROT(float, float, float);
  else if (tq == 0 && to == 1) SG_ROT(float, double, double);
  else if (tq == 1 && to == 1) SG_ROT(double, double, double);
  else if (tq == 1 && to == 0) SG_ROT(double, double, float);
  else return SG_ERR_ARG;
#undef SG_ROT
  SG_CHECK_LAUNCH();
  return SG_OK;
}
