// Batched block Krylov-Schur: many independent datasets embedded together.
//
// The datasets' matrices are stacked block-diagonally (rows roff[d]..roff[d+1]
// belong to dataset d, columns coff[d]..coff[d+1]), so the two SpMM passes of
// the Gram matvec are single launches of sg_spmm over the stacked CSR/CSC.
// The dense block operations need the dataset boundaries:
//   bproj    C_d = Q_dᵀ W_d   per-CTA partials over rows of ONE dataset
//            (cta_r0/cta_r1 ranges, CTAs of dataset d contiguous from
//            ds_cta[d]) + fixed-order reduction per dataset
//   bupdate  W_i -= Q_i C_d(i)
//   bchol    Cholesky of every dataset's Gram block (one warp per dataset)
//   brinv    W_i <- W_i R_d(i)⁻¹
//   bhblock  Rayleigh-quotient block + coupling into every dataset's H
//   brotate  out_i = Q_i Y_d(i)   (thick restart / Ritz vectors)
// Dataset of a row: binary search of roff (kept in shared memory).
// `active[d] == 0` freezes a converged dataset: its rows and blocks are left
// untouched by update/rinv (its SpMM rows still run; they are cheap to skip
// only by rebuilding the stacked matrix).
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kMaxDatasets = 4096;

__device__ __forceinline__ int find_ds(const int64_t* roff_s, int D, int64_t i) {
  int a = 0, b = D;  // last d with roff[d] <= i
  while (b - a > 1) {
    const int m = (a + b) >> 1;
    if (roff_s[m] <= i) a = m; else b = m;
  }
  return a;
}

template <typename T, int B, int CPT>
__global__ void __launch_bounds__(256)
bproj_partial(const int64_t* __restrict__ cta_r0, const int64_t* __restrict__ cta_r1, const int* __restrict__ cta_ds,
              const int* __restrict__ active, const T* __restrict__ Q, int64_t ldq, int ncols,
              const T* __restrict__ W, double* __restrict__ part) {
  __shared__ T ws[32][B];
  const int b = blockIdx.x;
  if (active && !active[cta_ds[b]]) return;  // frozen dataset: its C is not used
  const int64_t r0 = cta_r0[b], r1 = cta_r1[b];
  T acc[CPT][B];
#pragma unroll
  for (int q = 0; q < CPT; ++q)
#pragma unroll
    for (int c = 0; c < B; ++c) acc[q][c] = T(0);
  for (int64_t base = r0; base < r1; base += 32) {
    const int nr = (r1 - base) < 32 ? (int)(r1 - base) : 32;
    __syncthreads();
    for (int t = threadIdx.x; t < 32 * B; t += 256) {
      const int i = t / B, c = t % B;
      ws[i][c] = i < nr ? W[(base + i) * B + c] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < CPT; ++q) {
      const int p = threadIdx.x + q * 256;
      if (p < ncols) {
        // several rows' loads in flight, then their FMAs in row order
        constexpr int RU = B * CPT * (int)sizeof(T) >= 64 ? 2 : 8;
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
    const int p = threadIdx.x + q * 256;
    if (p < ncols) {
#pragma unroll
      for (int c = 0; c < B; ++c) part[((int64_t)b * ncols + p) * B + c] = (double)acc[q][c];
    }
  }
}

// C[d][t] = sum over the CTAs of dataset d of part[cta][t]  (t < ncols*B)
__global__ void bproj_reduce(int D, const int* __restrict__ ds_cta, int tot, const double* __restrict__ part,
                             double* __restrict__ C, int64_t cstride) {
  const int d = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= D || t >= tot) return;
  double s = 0.0;
  for (int b = ds_cta[d]; b < ds_cta[d + 1]; ++b) s += part[(int64_t)b * tot + t];
  C[(int64_t)d * cstride + t] = s;
}

template <typename T, int B>
__global__ void __launch_bounds__(256)
bupdate_kernel(int64_t nrows, const int64_t* __restrict__ roff, int D, const int* __restrict__ active,
               const T* __restrict__ Q, int64_t ldq, int ncols, const double* __restrict__ C, int64_t cstride,
               T* __restrict__ W) {
  __shared__ int64_t roff_s[kMaxDatasets + 1];
  for (int t = threadIdx.x; t <= D; t += blockDim.x) roff_s[t] = roff[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = gw; i < nrows; i += nw) {
    const int d = find_ds(roff_s, D, i);
    if (active && !active[d]) continue;
    const double* Cd = C + (int64_t)d * cstride;
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
#pragma unroll
          for (int c = 0; c < B; ++c) acc[c] = fma(qv[u], (T)Cd[p * B + c], acc[c]);
        }
      }
    }
    warp_colsum<T, B>(acc, lane);
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

// One warp per dataset: G_d = R_dᵀ R_d, Rinv_d = R_d⁻¹ (as chol_kernel).
__global__ void bchol_kernel(int B, int D, const int* __restrict__ active, const double* __restrict__ G,
                             double* __restrict__ R, double* __restrict__ Rinv, int* status, int* bad_ds) {
  __shared__ double r[32][33];
  __shared__ double x[32][33];  // x[i][j]: row i of column j of R^-1
  const int d = blockIdx.x;
  const int j = threadIdx.x;
  if (d >= D) return;
  const double* g = G + (int64_t)d * B * B;
  double* Ro = R + (int64_t)d * B * B;
  double* Ri = Rinv + (int64_t)d * B * B;
  if (active && !active[d]) {  // frozen: identity, so the caller's buffers stay defined
    if (j < B)
      for (int i = 0; i < B; ++i) { Ro[i * B + j] = i == j; Ri[i * B + j] = i == j; }
    return;
  }
  for (int i = 0; i < B; ++i) r[i][j] = 0.0;
  __syncwarp();
  bool fail = false;
  for (int k = 0; k < B; ++k) {
    if (j == k) {
      double s = g[k * B + k];
      for (int i = 0; i < k; ++i) s -= r[i][k] * r[i][k];
      const double gkk = g[k * B + k];
      if (!(s > 1e-28 * (gkk > 0 ? gkk : 1.0)) || !(s > 0.0)) { fail = true; s = 1.0; }
      r[k][k] = sqrt(s);
    }
    __syncwarp();
    const double piv = r[k][k];
    if (j > k && j < B) {
      double s = g[k * B + j];
      for (int i = 0; i < k; ++i) s -= r[i][k] * r[i][j];
      r[k][j] = s / piv;
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, fail) && j == 0) {
    atomicCAS(status, 0, SG_ERR_NUMERIC);
    if (bad_ds) atomicMin(bad_ds, d);
  }
  // back substitution, lane j builds column j of R^-1 in shared memory
  if (j < B) {
    for (int i = 0; i < B; ++i) x[i][j] = 0.0;
    x[j][j] = 1.0 / r[j][j];
    for (int i = j - 1; i >= 0; --i) {
      double s = 0.0;
      for (int t = i + 1; t <= j; ++t) s += r[i][t] * x[t][j];
      x[i][j] = -s / r[i][i];
    }
    for (int i = 0; i < B; ++i) {
      Ri[i * B + j] = i <= j ? x[i][j] : 0.0;
      Ro[i * B + j] = r[i][j];
    }
  }
}

template <typename T, int B>
__global__ void __launch_bounds__(256)
brinv_kernel(int64_t nrows, const int64_t* __restrict__ roff, int D, const int* __restrict__ active,
             const double* __restrict__ Rinv, T* __restrict__ W) {
  __shared__ int64_t roff_s[kMaxDatasets + 1];
  for (int t = threadIdx.x; t <= D; t += blockDim.x) roff_s[t] = roff[t];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  if constexpr (B <= 8) {  // thread per row: W[i,:] <- W[i,:] Rinv, column c over k = 0..c in order
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nrows;
         i += (int64_t)gridDim.x * blockDim.x) {
      const int d = find_ds(roff_s, D, i);
      if (active && !active[d]) continue;
      const double* ri = Rinv + (int64_t)d * B * B;
      T w[B], o[B];
#pragma unroll
      for (int k = 0; k < B; ++k) w[k] = W[i * B + k];
#pragma unroll
      for (int c = 0; c < B; ++c) {
        T s = T(0);
#pragma unroll
        for (int k = 0; k <= c; ++k) s = fma(w[k], (T)ri[k * B + c], s);
        o[c] = s;
      }
#pragma unroll
      for (int c = 0; c < B; ++c) W[i * B + c] = o[c];
    }
  } else {  // warp per row, lane c computes column c
    for (int64_t i = gw; i < nrows; i += nw) {
      const int d = find_ds(roff_s, D, i);
      if (active && !active[d]) continue;
      const double* ri = Rinv + (int64_t)d * B * B;
      const T w = lane < B ? W[i * B + lane] : T(0);
      T s = T(0);
#pragma unroll
      for (int k = 0; k < B; ++k) {
        const T wk = __shfl_sync(0xffffffffu, w, k);
        if (lane < B && k <= lane) s = fma(wk, (T)ri[k * B + lane], s);
      }
      if (lane < B) W[i * B + lane] = s;
    }
  }
}

__global__ void bhblock_kernel(int B, int D, const int* __restrict__ active, double* __restrict__ H, int64_t ldh,
                               int m0, const double* __restrict__ C1, const double* __restrict__ C2,
                               int64_t cstride, const double* __restrict__ R1, const double* __restrict__ R2,
                               double* __restrict__ Rout) {
  const int d = blockIdx.x;
  const int r = threadIdx.y, c = threadIdx.x;
  if (d >= D || r >= B || c >= B) return;
  if (active && !active[d]) return;
  double* Hd = H + (int64_t)d * ldh * ldh;
  const double* c1 = C1 + (int64_t)d * cstride;
  const double* c2 = C2 + (int64_t)d * cstride;
  const double d1 = c1[(int64_t)(m0 + r) * B + c] + c2[(int64_t)(m0 + r) * B + c];
  const double d2 = c1[(int64_t)(m0 + c) * B + r] + c2[(int64_t)(m0 + c) * B + r];
  Hd[(int64_t)(m0 + r) * ldh + m0 + c] = 0.5 * (d1 + d2);
  const double* r1 = R1 + (int64_t)d * B * B;
  const double* r2 = R2 + (int64_t)d * B * B;
  double s = 0.0;
  for (int k = 0; k < B; ++k) s += r2[r * B + k] * r1[k * B + c];
  Rout[(int64_t)d * B * B + r * B + c] = s;
  Hd[(int64_t)(m0 + B + r) * ldh + m0 + c] = s;
  Hd[(int64_t)(m0 + c) * ldh + m0 + B + r] = s;
}

// out_i[0:k] = Q_i[0:m] Y_d (Y: D x m x ldy, FP64); CTA -> rows of one dataset.
template <typename TQ, typename TA, typename TO>
__global__ void __launch_bounds__(256)
brotate_kernel(const int* __restrict__ cta_ds, const int64_t* __restrict__ cta_r0, const int64_t* __restrict__ cta_r1,
               const TQ* __restrict__ Q, int64_t ldq, int m, const double* __restrict__ Y, int64_t ldy,
               int64_t ystride, int k, TO* __restrict__ out, int64_t ldo) {
  extern __shared__ __align__(16) unsigned char sraw[];
  TA* ys = reinterpret_cast<TA*>(sraw);  // m x 32
  const int b = blockIdx.x;
  const int d = cta_ds[b];
  const double* Yd = Y + (int64_t)d * ystride;
  const int q0 = blockIdx.y * 32;
  for (int t = threadIdx.x; t < m * 32; t += blockDim.x) {
    const int p = t / 32, q = t % 32;
    ys[t] = (q0 + q < k) ? (TA)Yd[(int64_t)p * ldy + q0 + q] : TA(0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t r0 = cta_r0[b], r1 = cta_r1[b];
  for (int64_t i = r0 + w; i < r1; i += 8) {
    TA acc = TA(0);
    for (int p0 = 0; p0 < m; p0 += 32) {
      const TA qv = (p0 + lane < m) ? (TA)Q[i * ldq + p0 + lane] : TA(0);
      const int lim = min(32, m - p0);
      for (int t = 0; t < lim; ++t) acc = fma(__shfl_sync(0xffffffffu, qv, t), ys[(p0 + t) * 32 + lane], acc);
    }
    if (q0 + lane < k) out[i * ldo + q0 + lane] = (TO)acc;
  }
}

int nsm() {
  int dev = 0, s = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
  return s > 0 ? s : 1;
}

template <typename T, int B>
int bproj_t(int ncta, const int64_t* r0, const int64_t* r1, const int* cta_ds, const int* active, const int* ds_cta,
            int D, const T* Q, int64_t ldq, int ncols, const T* W, double* part, double* C, int64_t cstride,
            cudaStream_t s) {
  constexpr int kSlice = B * (int)sizeof(T) >= 128 ? 256 : 512;  // two thread columns only while they fit
  for (int c0 = 0; c0 < ncols; c0 += kSlice) {
    const int nc = ncols - c0 < kSlice ? ncols - c0 : kSlice;
    if constexpr (kSlice > 256) {
      if (nc > 256) bproj_partial<T, B, 2><<<ncta, 256, 0, s>>>(r0, r1, cta_ds, active, Q + c0, ldq, nc, W, part);
      else bproj_partial<T, B, 1><<<ncta, 256, 0, s>>>(r0, r1, cta_ds, active, Q + c0, ldq, nc, W, part);
    } else {
      bproj_partial<T, B, 1><<<ncta, 256, 0, s>>>(r0, r1, cta_ds, active, Q + c0, ldq, nc, W, part);
    }
    SG_CHECK_LAUNCH();
    const int tot = nc * B;
    dim3 g((tot + 255) / 256, D);
    bproj_reduce<<<g, 256, 0, s>>>(D, ds_cta, tot, part, C + (int64_t)c0 * B, cstride);
    SG_CHECK_LAUNCH();
  }
  return SG_OK;
}

}  // namespace
}  // namespace sg

using namespace sg;

#define SG_BDISPATCH(FN, ...)                        \
  switch (block) {                                   \
    case 4: return FN<T, 4>(__VA_ARGS__);            \
    case 8: return FN<T, 8>(__VA_ARGS__);            \
    case 16: return FN<T, 16>(__VA_ARGS__);          \
    case 32: return FN<T, 32>(__VA_ARGS__);          \
    default: return SG_ERR_ARG;                      \
  }

template <typename T>
static int bproj_any(int block, int ncta, const int64_t* r0, const int64_t* r1, const int* cta_ds, const int* active,
                     const int* ds_cta, int D, const T* Q, int64_t ldq, int ncols, const T* W, double* part, double* C,
                     int64_t cstride, cudaStream_t s) {
  SG_BDISPATCH(bproj_t, ncta, r0, r1, cta_ds, active, ds_cta, D, Q, ldq, ncols, W, part, C, cstride, s)
}

extern "C" int sg_bblock_proj(int dtype, int block, int D, int ncta, const int* ds_cta, const int* cta_ds,
                              const int* active, const int64_t* cta_r0, const int64_t* cta_r1, const void* Q,
                              int64_t ldq, int ncols, const void* W, double* part, double* C, int64_t cstride,
                              void* stream) {
  if (D <= 0 || D > kMaxDatasets || ncta <= 0 || ncols <= 0 || cstride < (int64_t)ncols * block) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (dtype == 0)
    return bproj_any<float>(block, ncta, cta_r0, cta_r1, cta_ds, active, ds_cta, D, (const float*)Q, ldq, ncols,
                            (const float*)W, part, C, cstride, s);
  if (dtype == 1)
    return bproj_any<double>(block, ncta, cta_r0, cta_r1, cta_ds, active, ds_cta, D, (const double*)Q, ldq, ncols,
                             (const double*)W, part, C, cstride, s);
  return SG_ERR_ARG;
}

// mask[i] = active[dataset of i] for i < n (offsets off[D+1]).
__global__ void bmask_kernel(int64_t n, int D, const int64_t* __restrict__ off, const int* __restrict__ active,
                             unsigned char* __restrict__ mask) {
  __shared__ int64_t off_s[kMaxDatasets + 1];
  for (int t = threadIdx.x; t <= D; t += blockDim.x) off_s[t] = off[t];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    mask[i] = active[find_ds(off_s, D, i)] ? 1 : 0;
}

extern "C" int sg_bmask(int64_t n, int D, const int64_t* off, const int* active, unsigned char* mask, void* stream) {
  if (n <= 0 || D <= 0 || D > kMaxDatasets) return SG_ERR_ARG;
  bmask_kernel<<<grid_for(n, 256, 8 * nsm()), 256, 0, as_stream(stream)>>>(n, D, off, active, mask);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_bblock_update(int dtype, int block, int64_t nrows, int D, const int64_t* roff, const int* active,
                                const void* Q, int64_t ldq, int ncols, const double* C, int64_t cstride, void* W,
                                void* stream) {
  if (D <= 0 || D > kMaxDatasets || nrows <= 0 || ncols <= 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int grid = grid_for(nrows * 32, 256, 8 * nsm());
#define SG_BU(T, BB)                                                                                             \
  case BB:                                                                                                      \
    bupdate_kernel<T, BB><<<grid, 256, 0, s>>>(nrows, roff, D, active, (const T*)Q, ldq, ncols, C, cstride,     \
                                              (T*)W);                                                          \
    break;
  if (dtype == 0) {
    switch (block) { SG_BU(float, 4) SG_BU(float, 8) SG_BU(float, 16) SG_BU(float, 32) default: return SG_ERR_ARG; }
  } else if (dtype == 1) {
    switch (block) { SG_BU(double, 4) SG_BU(double, 8) SG_BU(double, 16) SG_BU(double, 32) default: return SG_ERR_ARG; }
  } else {
    return SG_ERR_ARG;
  }
#undef SG_BU
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// One batched Cholesky-QR pass over every dataset's block.
extern "C" int sg_bblock_cholqr(int dtype, int block, int64_t nrows, int D, const int64_t* roff, const int* active,
                                int ncta, const int* ds_cta, const int* cta_ds, const int64_t* cta_r0,
                                const int64_t* cta_r1, void* W, double* part, double* G, double* R, double* Rinv,
                                int* status, int* bad_ds, void* stream) {
  if (block < 1 || block > 32) return SG_ERR_ARG;
  int e = sg_bblock_proj(dtype, block, D, ncta, ds_cta, cta_ds, active, cta_r0, cta_r1, W, block, block, W, part, G,
                         (int64_t)block * block, stream);
  if (e) return e;
  cudaStream_t s = as_stream(stream);
  bchol_kernel<<<D, 32, 0, s>>>(block, D, active, G, R, Rinv, status, bad_ds);
  SG_CHECK_LAUNCH();
  const int grid = grid_for(nrows * 32, 256, 8 * nsm());
#define SG_BR(T, BB) \
  case BB: brinv_kernel<T, BB><<<grid, 256, 0, s>>>(nrows, roff, D, active, Rinv, (T*)W); break;
  if (dtype == 0) {
    switch (block) { SG_BR(float, 4) SG_BR(float, 8) SG_BR(float, 16) SG_BR(float, 32) default: return SG_ERR_ARG; }
  } else if (dtype == 1) {
    switch (block) { SG_BR(double, 4) SG_BR(double, 8) SG_BR(double, 16) SG_BR(double, 32) default: return SG_ERR_ARG; }
  } else {
    return SG_ERR_ARG;
  }
#undef SG_BR
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_blanczos_hblock(int block, int D, const int* active, double* H, int64_t ldh, int m0,
                                  const double* C1, const double* C2, int64_t cstride, const double* R1,
                                  const double* R2, double* Rout, void* stream) {
  if (block < 1 || block > 32 || D <= 0 || m0 < 0) return SG_ERR_ARG;
  bhblock_kernel<<<D, dim3(block, block), 0, as_stream(stream)>>>(block, D, active, H, ldh, m0, C1, C2, cstride, R1,
                                                                  R2, Rout);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_bbasis_rotate(int tq, int to, int ncta, const int* cta_ds, const int64_t* cta_r0,
                                const int64_t* cta_r1, const void* Q, int64_t ldq, int m, const double* Y, int64_t ldy,
                                int64_t ystride, int k, void* out, int64_t ldo, void* stream) {
  if (ncta <= 0 || m <= 0 || k <= 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  dim3 grid(ncta, (k + 31) / 32);
  const bool wide = tq == 1 || to == 1;
  const size_t smem = (size_t)m * 32 * (wide ? sizeof(double) : sizeof(float));
  if (smem > 200 * 1024) return SG_ERR_ARG;
#define SG_BROT(TQ, TA, TO)                                                                                  \
  do {                                                                                                       \
    if (smem > 48 * 1024 &&                                                                                  \
        cudaFuncSetAttribute(brotate_kernel<TQ, TA, TO>, cudaFuncAttributeMaxDynamicSharedMemorySize,        \
                             200 * 1024) != cudaSuccess)                                                     \
      return SG_ERR_CUDA;                                                                                    \
    brotate_kernel<TQ, TA, TO><<<grid, 256, smem, s>>>(cta_ds, cta_r0, cta_r1, (const TQ*)Q, ldq, m, Y, ldy, \
                                                       ystride, k, (TO*)out, ldo);                           \
  } while (0)
  if (tq == 0 && to == 0) SG_BROT(float, float, float);
  else if (tq == 0 && to == 1) SG_BROT(float, double, double);
  else if (tq == 1 && to == 1) SG_BROT(double, double, double);
  else return SG_ERR_ARG;
#undef SG_BROT
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// Per-dataset IDF on stacked columns (embedding.rs:269-286 per dataset):
// w_j = ln(n_d / c_j) with the reference's count rules, all-equal -> 1.
__global__ void bidf_minmax(int64_t m, const int64_t* __restrict__ colptr, int D, const int64_t* __restrict__ coff,
                            unsigned long long* __restrict__ mm) {
  __shared__ int64_t coff_s[kMaxDatasets + 1];
  for (int t = threadIdx.x; t <= D; t += blockDim.x) coff_s[t] = coff[t];
  __syncthreads();
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const int d = find_ds(coff_s, D, j);
    const unsigned long long c = (unsigned long long)(colptr[j + 1] - colptr[j]);
    atomicMin(mm + 2 * d, c);
    atomicMax(mm + 2 * d + 1, c);
  }
}

__global__ void bidf_init(int D, unsigned long long* mm) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < D; d += gridDim.x * blockDim.x) {
    mm[2 * d] = ~0ull;
    mm[2 * d + 1] = 0ull;
  }
}

__global__ void bidf_kernel(int64_t m, const int64_t* __restrict__ colptr, int D, const int64_t* __restrict__ coff,
                            const int64_t* __restrict__ roff, const unsigned long long* __restrict__ mm,
                            double* __restrict__ w) {
  __shared__ int64_t coff_s[kMaxDatasets + 1];
  for (int t = threadIdx.x; t <= D; t += blockDim.x) coff_s[t] = coff[t];
  __syncthreads();
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const int d = find_ds(coff_s, D, j);
    if (mm[2 * d] == mm[2 * d + 1]) { w[j] = 1.0; continue; }
    const double dn = (double)(roff[d + 1] - roff[d]);
    double c = (double)(colptr[j + 1] - colptr[j]);
    if (c == 0.0) c = 1.0;
    else if (c == dn) c = dn - 1.0;
    w[j] = log(dn / c);
  }
}

extern "C" int sg_bidf(int64_t m, const int64_t* colptr, int D, const int64_t* coff, const int64_t* roff,
                       unsigned long long* minmax, double* w, void* stream) {
  if (m <= 0 || D <= 0 || D > kMaxDatasets) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  bidf_init<<<(D + 255) / 256, 256, 0, s>>>(D, minmax);
  const int g = grid_for(m, 256, 8 * nsm());
  bidf_minmax<<<g, 256, 0, s>>>(m, colptr, D, coff, minmax);
  bidf_kernel<<<g, 256, 0, s>>>(m, colptr, D, coff, roff, minmax, w);
  SG_CHECK_LAUNCH();
  return SG_OK;
}
