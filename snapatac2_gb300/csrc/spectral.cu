// Matrix-free cosine spectral operator: feature selection, deterministic CSR
// transpose, IDF weights, row normalisation, degree, and the two CSR SpMM
// kernels of the Gram product.
//
// Reference arithmetic (snapatac2-python/src/embedding.rs):
//   idf        269-286   w_j = ln(n / c_j), c_j = nnz of column j (0 -> 1,
//                        n -> n-1; all counts equal -> w = 1)
//   normalize  315-326   Xn = diag(1/||(XW)_i||) X W
//   degree     139-152   colsum = 1ᵀXn, d = Xn colsum, D⁻¹ = 1/(d - 1)
//   eigen      155-171   operator v -> X̂ (X̂ᵀ v) - D⁻¹ v, X̂ = diag(sqrt(D⁻¹)) Xn
// With a_i = sqrt(D⁻¹_i)/||(XW)_i|| the operator is
//   A v = a ⊙ (X (w² ⊙ (Xᵀ (a ⊙ v)))) - D⁻¹ ⊙ v
// so X is kept as an index-only pattern (or with its integer counts) and the
// scalings are folded into the SpMM prologue/epilogue.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

// ---------------------------------------------------------------------------
// column selection: keep entries whose column maps to >= 0, renumbered
// ---------------------------------------------------------------------------
__global__ void select_count(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                             const int32_t* __restrict__ colmap, int64_t* __restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w; r < n; r += nw) {
    int64_t c = 0;
    for (int64_t e = ptr[r] + lane; e < ptr[r + 1]; e += 32) c += colmap[idx[e]] >= 0;
    for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) cnt[r + 1] = c;
  }
}

__global__ void select_fill(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                            const float* __restrict__ val, const int32_t* __restrict__ colmap,
                            const int64_t* __restrict__ optr, int32_t* __restrict__ oidx,
                            float* __restrict__ oval) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = w; r < n; r += nw) {
    int64_t o = optr[r];
    const int64_t b = ptr[r], e = ptr[r + 1];
    for (int64_t k0 = b; k0 < e; k0 += 32) {
      const int64_t k = k0 + lane;
      int nc = -1;
      if (k < e) nc = colmap[idx[k]];
      const unsigned keep = __ballot_sync(0xffffffffu, nc >= 0);
      if (nc >= 0) {
        const int64_t p = o + __popc(keep & lanemask_lt());
        oidx[p] = nc;
        if (oval) oval[p] = val[k];
      }
      o += __popc(keep);
    }
  }
}

// ---------------------------------------------------------------------------
// deterministic transpose (CSR -> CSC) with rows ascending inside each column
//
// Columns are cut into panels of kTrPanel columns so that a CTA keeps the
// counters / cursors of one panel in shared memory.  seg[r][p] is the offset
// (from the row start) of row r's first entry in panel p (rows are sorted, so
// a row's entries of one panel are contiguous).  Rows are split into nblk row
// blocks; for every (row block, panel):
//   count : shared-memory histogram of the panel's columns, written to
//           cnt[b][col] (coalesced);
//   offsets: cnt[b][col] <- sum over earlier row blocks (column-wise scan);
//   fill  : the CTA walks its rows in order and appends each row index to
//           its column (one entry per column per row, so no two threads touch
//           the same cursor inside a row; rows are separated by a barrier).
// Row order inside every column is therefore ascending and the result is
// identical run to run.
// ---------------------------------------------------------------------------
constexpr int kTrPanel = 16384;

__global__ void seg_kernel(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx, int pw,
                           int P, int64_t m, int32_t* __restrict__ seg, int* status) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < n; r += nw) {
    const int64_t s = ptr[r], e = ptr[r + 1];
    int32_t* sg = seg + r * (int64_t)(P + 1);
    const int len = (int)(e - s);
    for (int64_t k0 = s; k0 < e + 1; k0 += 32) {
      const int64_t k = k0 + lane;
      if (k > e) continue;
      // panel of this entry (P for the end sentinel) and of the previous one
      int pc = P, pp = -1;
      if (k < e) {
        const int c = idx[k];
        if (c < 0 || c >= m || (k > s && idx[k - 1] >= c)) {  // need sorted, unique, in range
          report_error(status, nullptr, SG_ERR_ARG, 0);
          pc = P;
        } else {
          pc = c / pw;
        }
      }
      if (k > s) {
        const int cprev = idx[k - 1];
        pp = (cprev >= 0 && cprev < m) ? cprev / pw : P;
      }
      for (int p = pp + 1; p <= pc && p <= P; ++p) sg[p] = (int32_t)(k - s);
    }
    if (len == 0 && lane == 0)
      for (int p = 0; p <= P; ++p) sg[p] = 0;
  }
}

__global__ void __launch_bounds__(512)
tr_count(int64_t n, int64_t m, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
         const int32_t* __restrict__ seg, int P, int nblk, int32_t* __restrict__ cnt, const int* status) {
  __shared__ int32_t c_s[kTrPanel];
  if (*status) return;  // invalid column indices: seg is not trustworthy
  const int b = blockIdx.x, p = blockIdx.y;
  const int64_t r0 = n * b / nblk, r1 = n * (b + 1) / nblk;
  const int64_t col0 = (int64_t)p * kTrPanel;
  const int width = (int)min((int64_t)kTrPanel, m - col0);
  for (int j = threadIdx.x; j < width; j += blockDim.x) c_s[j] = 0;
  __syncthreads();
  for (int64_t r = r0; r < r1; ++r) {
    const int32_t* sg = seg + r * (int64_t)(P + 1);
    const int64_t s = ptr[r] + sg[p], e = ptr[r] + sg[p + 1];
    for (int64_t k = s + threadIdx.x; k < e; k += blockDim.x) atomicAdd(&c_s[idx[k] - col0], 1);
  }
  __syncthreads();
  int32_t* out = cnt + (int64_t)b * m + col0;
  for (int j = threadIdx.x; j < width; j += blockDim.x) out[j] = c_s[j];
}

// colptr[j+1] = total count of column j
__global__ void tr_total(int64_t m, int nblk, const int32_t* __restrict__ cnt, int64_t* __restrict__ colptr) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    int64_t t = 0;
    for (int b = 0; b < nblk; ++b) t += cnt[(int64_t)b * m + j];
    colptr[j + 1] = t;
    if (j == 0) colptr[0] = 0;
  }
}

// cnt[b][j] <- sum_{b' < b} cnt[b'][j]  (row block b's offset inside column j)
__global__ void tr_offsets(int64_t m, int nblk, int32_t* __restrict__ cnt) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    int64_t run = 0;
    for (int b = 0; b < nblk; ++b) {
      const int64_t c = cnt[(int64_t)b * m + j];
      cnt[(int64_t)b * m + j] = (int32_t)run;
      run += c;
    }
  }
}

__global__ void __launch_bounds__(512)
tr_fill(int64_t n, int64_t m, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
        const float* __restrict__ val, const int32_t* __restrict__ seg, int P, int nblk,
        const int32_t* __restrict__ cnt, const int64_t* __restrict__ colptr, int32_t* __restrict__ rowidx,
        float* __restrict__ cval, const int* status) {
  __shared__ int32_t cur[kTrPanel];
  if (*status) return;
  const int b = blockIdx.x, p = blockIdx.y;
  const int64_t r0 = n * b / nblk, r1 = n * (b + 1) / nblk;
  const int64_t col0 = (int64_t)p * kTrPanel;
  const int width = (int)min((int64_t)kTrPanel, m - col0);
  const int32_t* in = cnt + (int64_t)b * m + col0;
  for (int j = threadIdx.x; j < width; j += blockDim.x) cur[j] = in[j];
  __syncthreads();
  for (int64_t r = r0; r < r1; ++r) {
    const int32_t* sg = seg + r * (int64_t)(P + 1);
    const int64_t s = ptr[r] + sg[p], e = ptr[r] + sg[p + 1];
    for (int64_t k = s + threadIdx.x; k < e; k += blockDim.x) {
      const int c = idx[k];
      const int j = c - (int)col0;
      const int pos = cur[j];
      cur[j] = pos + 1;
      const int64_t dst = colptr[c] + pos;
      rowidx[dst] = (int32_t)r;
      if (cval) cval[dst] = val[k];
    }
    __syncthreads();  // the next row may touch the same columns
  }
}

// ---------------------------------------------------------------------------
// IDF weights, row norms, degree (FP64, as the reference)
// ---------------------------------------------------------------------------
__global__ void colcount_minmax(int64_t m, const int64_t* __restrict__ colptr, unsigned long long* mm) {
  unsigned long long lo = ~0ull, hi = 0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    unsigned long long c = (unsigned long long)(colptr[j + 1] - colptr[j]);
    lo = min(lo, c);
    hi = max(hi, c);
  }
  for (int o = 16; o; o >>= 1) {
    lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mm, lo);
    atomicMax(mm + 1, hi);
  }
}

__global__ void init_minmax(unsigned long long* mm) {
  mm[0] = ~0ull;
  mm[1] = 0ull;
}

__global__ void idf_kernel(int64_t n, int64_t m, const int64_t* __restrict__ colptr,
                           const unsigned long long* __restrict__ mm, double* __restrict__ w) {
  const bool equal = mm[0] == mm[1];
  const double dn = (double)n;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    if (equal) { w[j] = 1.0; continue; }
    double c = (double)(colptr[j + 1] - colptr[j]);
    if (c == 0.0) c = 1.0;
    else if (c == dn) c = dn - 1.0;
    w[j] = log(dn / c);
  }
}

// rinv_i = 1 / ||(x_i ⊙ w)||_2
__global__ void rownorm_kernel(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                               const float* __restrict__ val, const double* __restrict__ w,
                               double* __restrict__ rinv, int* status, unsigned long long* bad) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < n; r += nw) {
    double s = 0.0;
    for (int64_t k = ptr[r] + lane; k < ptr[r + 1]; k += 32) {
      double x = w[idx[k]];
      if (val) x *= (double)val[k];
      s = fma(x, x, s);
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      if (!(s > 0.0)) report_error(status, bad, SG_ERR_NUMERIC, (unsigned long long)r);
      rinv[r] = 1.0 / sqrt(s);
    }
  }
}

// colsum_j = w_j * sum_{i in col j} x_ij rinv_i   (CSC gather)
__global__ void colsum_kernel(int64_t m, const int64_t* __restrict__ cptr, const int32_t* __restrict__ ridx,
                              const float* __restrict__ cval, const double* __restrict__ w,
                              const double* __restrict__ rinv, double* __restrict__ colsum) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = gw; j < m; j += nw) {
    double s = 0.0;
    for (int64_t k = cptr[j] + lane; k < cptr[j + 1]; k += 32) {
      double x = rinv[ridx[k]];
      if (cval) x *= (double)cval[k];
      s += x;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) colsum[j] = s * w[j];
  }
}

// d_i = rinv_i * sum_j x_ij w_j colsum_j ; dinv = 1/(d-1) ; a = rinv*sqrt(dinv)
__global__ void degree_kernel(int64_t n, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
                              const float* __restrict__ val, const double* __restrict__ w,
                              const double* __restrict__ colsum, const double* __restrict__ rinv,
                              double* __restrict__ a, double* __restrict__ dinv, float* __restrict__ a32,
                              float* __restrict__ dinv32, int* status, unsigned long long* bad) {
  const int lane = threadIdx.x & 31;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = gw; r < n; r += nw) {
    double s = 0.0;
    for (int64_t k = ptr[r] + lane; k < ptr[r + 1]; k += 32) {
      const int j = idx[k];
      double x = w[j] * colsum[j];
      if (val) x *= (double)val[k];
      s += x;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
      const double d = s * rinv[r];
      const double di = 1.0 / (d - 1.0);
      if (!(di > 0.0) || isinf(di)) report_error(status, bad, SG_ERR_NUMERIC, (unsigned long long)r);
      const double ai = rinv[r] * sqrt(di);
      a[r] = ai;
      dinv[r] = di;
      if (a32) a32[r] = (float)ai;
      if (dinv32) dinv32[r] = (float)di;
    }
  }
}

__global__ void square_weights(int64_t m, const double* __restrict__ w, double* __restrict__ w2,
                               float* __restrict__ w2f) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const double v = w[j] * w[j];
    w2[j] = v;
    if (w2f) w2f[j] = (float)v;
  }
}

// ---------------------------------------------------------------------------
// CSR SpMM over a block of B dense columns:
//   out[r,:] = s_r * sum_{e in row r} x_e * in[col_e,:]  (- d_r * y[r,:])
// One warp per row.  The B values of a gathered row are split into 16-byte
// vectors, LPN lanes per nonzero, so each warp step gathers 32/LPN rows with
// coalesced 128-bit loads; the 32 column indices of a chunk are read once
// (one coalesced 128-byte load) and broadcast by shuffles.  Partial sums are
// combined by a fixed xor-shuffle tree: results are deterministic.
// ---------------------------------------------------------------------------
// Variants (same arithmetic, same result, picked by the autotuner): bits 0-1
// select 1, 2, 4 or 8 chunks of 32 column indices in flight per iteration
// (more gathers outstanding per lane against fewer resident warps); bit 2
// sends the gathers through L2 only (ld.global.cg).
template <typename VT>
__device__ __forceinline__ VT gather16(const VT* p, bool l2only) {
  return l2only ? __ldcg(p) : __ldg(p);
}

// DYN: a persistent grid whose warps take kDynRows rows at a time from an
// atomic counter (zeroed by the host before the launch), so that the long
// rows of a skewed matrix do not leave a tail of idle SMs; each row is still
// summed by one warp in the same order (same result as the static schedule).
constexpr int kDynRows = 4;
// With `order` the counter walks positions instead of rows: order[p] is the
// row at position p (-1: none), laid out by sg_row_order so that the longest
// rows are taken first, one per 4-row fetch (longest-first scheduling: the
// last rows to finish are short ones).  Each row is still summed by one warp
// in the same order: the result does not change.

template <typename T, int B, bool VALUED, bool SHIFT, int VAR, bool DYN = false>
__global__ void __launch_bounds__(256)
spmm_kernel(int64_t rows, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
            const float* __restrict__ val, const T* __restrict__ in, T* __restrict__ out,
            const T* __restrict__ scale, const T* __restrict__ dshift, const T* __restrict__ y,
            const unsigned char* __restrict__ row_mask, unsigned int* __restrict__ counter = nullptr,
            const int32_t* __restrict__ order = nullptr) {
  using VT = typename V16<T>::type;
  constexpr int VW = V16<T>::n;
  constexpr int LPN = B / VW;          // lanes per nonzero
  constexpr int NPS = 32 / LPN;        // nonzeros per warp step
  constexpr int CH = 1 << (VAR & 3);   // 32-index chunks per iteration
  constexpr bool L2ONLY = (VAR & 4) != 0;
  constexpr bool STREAM = false;
  static_assert(B % VW == 0 && LPN >= 1 && LPN <= 32, "unsupported block width");
  const int lane = threadIdx.x & 31;
  const int sub = lane % LPN, slot = lane / LPN;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t r = DYN ? 0 : gw, rend = DYN ? 0 : rows;
  while (true) {
    if (DYN) {
      if (r >= rend) {  // next chunk of rows for this warp
        unsigned int c0 = 0;
        if (lane == 0) c0 = atomicAdd(counter, (unsigned int)kDynRows);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        r = c0;
        rend = r + kDynRows < rows ? r + kDynRows : rows;
        if (r >= rows) break;
      }
    } else if (r >= rows) {
      break;
    }
    int64_t rr = r;
    r += DYN ? 1 : nw;
    if (DYN && order) {  // position -> row (-1: no row at this position)
      rr = order[rr];
      if (rr < 0) continue;
    }
    if (row_mask && !row_mask[rr]) continue;  // frozen row (warp-uniform)
    const int64_t s = ptr[rr], e = ptr[rr + 1];
    VT acc = V16<T>::zero();
    for (int64_t base = s; base < e; base += 32 * CH) {
      int ci[CH];
      float cv[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int64_t k = base + c * 32 + lane;
        ci[c] = k < e ? (STREAM ? __ldcs(idx + k) : __ldg(idx + k)) : -1;
        cv[c] = (VALUED && k < e) ? (STREAM ? __ldcs(val + k) : __ldg(val + k)) : 1.0f;
      }
      VT g[CH * LPN];
      float gv[CH * LPN];
#pragma unroll
      for (int c = 0; c < CH; ++c)
#pragma unroll
        for (int j = 0; j < LPN; ++j) {
          const int col = __shfl_sync(0xffffffffu, ci[c], j * NPS + slot);
          if (VALUED) gv[c * LPN + j] = __shfl_sync(0xffffffffu, cv[c], j * NPS + slot);
          g[c * LPN + j] = col >= 0 ? gather16(reinterpret_cast<const VT*>(in + (int64_t)col * B) + sub, L2ONLY)
                                    : V16<T>::zero();
        }
#pragma unroll
      for (int t = 0; t < CH * LPN; ++t) {
        if (VALUED) V16<T>::fma(acc, (T)gv[t], g[t]);
        else V16<T>::add(acc, g[t]);
      }
    }
#pragma unroll
    for (int o = LPN; o < 32; o <<= 1) V16<T>::add(acc, V16<T>::shfl_xor(acc, o));
    if (slot == 0) {
      const T sc = scale[rr];
      T* op = out + rr * B + sub * VW;
      const T* a = reinterpret_cast<const T*>(&acc);
      VT o;
      T* ov = reinterpret_cast<T*>(&o);
      if (SHIFT) {
        const T d = dshift[rr];
        const T* yp = y + rr * B + sub * VW;
#pragma unroll
        for (int q = 0; q < VW; ++q) ov[q] = sc * a[q] - d * yp[q];
      } else {
#pragma unroll
        for (int q = 0; q < VW; ++q) ov[q] = sc * a[q];
      }
      *reinterpret_cast<VT*>(op) = o;
    }
  }
}

constexpr int kSpmmVariants = 8;

template <typename T, int B, int VAR>
void launch_spmm_v(int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val, const T* in, T* out,
                   const T* scale, const T* dshift, const T* y, int grid, cudaStream_t s, const unsigned char* mk) {
  if (val) {
    if (dshift) spmm_kernel<T, B, true, true, VAR><<<grid, 256, 0, s>>>(rows, ptr, idx, val, in, out, scale, dshift, y, mk);
    else spmm_kernel<T, B, true, false, VAR><<<grid, 256, 0, s>>>(rows, ptr, idx, val, in, out, scale, dshift, y, mk);
  } else {
    if (dshift) spmm_kernel<T, B, false, true, VAR><<<grid, 256, 0, s>>>(rows, ptr, idx, val, in, out, scale, dshift, y, mk);
    else spmm_kernel<T, B, false, false, VAR><<<grid, 256, 0, s>>>(rows, ptr, idx, val, in, out, scale, dshift, y, mk);
  }
}

template <typename T, int B>
int launch_spmm_t(int variant, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val, const T* in,
                  T* out, const T* scale, const T* dshift, const T* y, int grid, cudaStream_t s,
                  const unsigned char* mk) {
  switch (variant) {
    case 0: launch_spmm_v<T, B, 0>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 1: launch_spmm_v<T, B, 1>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 2: launch_spmm_v<T, B, 2>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 3: launch_spmm_v<T, B, 3>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 4: launch_spmm_v<T, B, 4>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 5: launch_spmm_v<T, B, 5>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 6: launch_spmm_v<T, B, 6>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    case 7: launch_spmm_v<T, B, 7>(rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk); break;
    default: return SG_ERR_ARG;
  }
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

template <typename T>
int launch_spmm(int variant, int B, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
                const T* in, T* out, const T* scale, const T* dshift, const T* y, int grid, cudaStream_t s,
                const unsigned char* mk) {
  switch (B) {
    case 4: return launch_spmm_t<T, 4>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk);
    case 8: return launch_spmm_t<T, 8>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk);
    case 16: return launch_spmm_t<T, 16>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk);
    case 32: return launch_spmm_t<T, 32>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, grid, s, mk);
    default: return SG_ERR_ARG;
  }
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_csr_select_cols(int64_t n, const int64_t* indptr, const int32_t* indices, const float* values,
                                  const int32_t* colmap, int64_t* out_indptr, int32_t* out_indices,
                                  float* out_values, void* scan_scratch, void* stream) {
  if (n < 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (n == 0) return cudaMemsetAsync(out_indptr, 0, sizeof(int64_t), s) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
  const int grid = grid_for(n * 32, 256, 8 * sm_count() * 8);
  if (cudaMemsetAsync(out_indptr, 0, sizeof(int64_t), s) != cudaSuccess) return SG_ERR_CUDA;
  select_count<<<grid, 256, 0, s>>>(n, indptr, indices, colmap, out_indptr);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(out_indptr + 1, n, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  select_fill<<<grid, 256, 0, s>>>(n, indptr, indices, values, colmap, out_indptr, out_indices, out_values);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_transpose_blocks(void) { return 2 * sm_count(); }

extern "C" int64_t sg_transpose_work_bytes(int64_t n, int64_t m, int nblk) {
  if (n < 0 || m <= 0 || nblk <= 0) return -1;
  const int64_t P = (m + kTrPanel - 1) / kTrPanel;
  const int64_t cnt = (int64_t)nblk * m * 4;
  return (cnt + 255) / 256 * 256 + n * (P + 1) * 4;
}

extern "C" int sg_csr_transpose(int64_t n, int64_t m, const int64_t* indptr, const int32_t* indices,
                                const float* values, int nblk, void* work, int64_t work_bytes, int64_t* colptr,
                                int32_t* rowidx, float* cvalues, void* scan_scratch, int* status, void* stream) {
  if (n <= 0 || m <= 0 || nblk <= 0 || m > 0x7fffffffLL || n > 0x7fffffffLL) return SG_ERR_ARG;
  if (work_bytes < sg_transpose_work_bytes(n, m, nblk) || ((uintptr_t)work & 255u)) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  const int P = (int)((m + kTrPanel - 1) / kTrPanel);
  int32_t* cnt = reinterpret_cast<int32_t*>(work);
  int32_t* seg = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(work) + ((int64_t)nblk * m * 4 + 255) / 256 * 256);
  seg_kernel<<<grid_for(n * 32, 256, 8 * sm_count() * 4), 256, 0, s>>>(n, indptr, indices, kTrPanel, P, m, seg,
                                                                        status);
  SG_CHECK_LAUNCH();
  dim3 g2(nblk, P);
  tr_count<<<g2, 512, 0, s>>>(n, m, indptr, indices, seg, P, nblk, cnt, status);
  SG_CHECK_LAUNCH();
  const int g = grid_for(m, 256, 4096);
  tr_total<<<g, 256, 0, s>>>(m, nblk, cnt, colptr);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(colptr + 1, m, scan_scratch, s) != cudaSuccess) return SG_ERR_CUDA;
  tr_offsets<<<g, 256, 0, s>>>(m, nblk, cnt);
  SG_CHECK_LAUNCH();
  tr_fill<<<g2, 512, 0, s>>>(n, m, indptr, indices, values, seg, P, nblk, cnt, colptr, rowidx, cvalues, status);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_spectral_prepare(int64_t n, int64_t m, const int64_t* indptr, const int32_t* indices,
                                   const float* values, const int64_t* colptr, const int32_t* rowidx,
                                   const float* cvalues, const double* feature_weights, double* w,
                                   double* w2, float* w2_32, double* rinv, double* colsum, double* a,
                                   double* dinv, float* a32, float* dinv32, unsigned long long* minmax,
                                   int* status, unsigned long long* bad, void* stream) {
  if (n <= 0 || m <= 0) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int sms = sm_count();
  const int gm = grid_for(m, 256, 8 * sms);
  const int gw_rows = grid_for(n * 32, 256, 8 * sms * 4);
  const int gw_cols = grid_for(m * 32, 256, 8 * sms * 4);
  if (feature_weights) {
    if (cudaMemcpyAsync(w, feature_weights, (size_t)m * sizeof(double), cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return SG_ERR_CUDA;
  } else {
    init_minmax<<<1, 1, 0, s>>>(minmax);
    colcount_minmax<<<gm, 256, 0, s>>>(m, colptr, minmax);
    SG_CHECK_LAUNCH();
    idf_kernel<<<gm, 256, 0, s>>>(n, m, colptr, minmax, w);
    SG_CHECK_LAUNCH();
  }
  square_weights<<<gm, 256, 0, s>>>(m, w, w2, w2_32);
  rownorm_kernel<<<gw_rows, 256, 0, s>>>(n, indptr, indices, values, w, rinv, status, bad);
  colsum_kernel<<<gw_cols, 256, 0, s>>>(m, colptr, rowidx, cvalues, w, rinv, colsum);
  degree_kernel<<<gw_rows, 256, 0, s>>>(n, indptr, indices, values, w, colsum, rinv, a, dinv, a32, dinv32,
                                        status, bad);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

template <int B, int VAR>
int launch_spmm_dyn_v(int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val, const float* in,
                      float* out, const float* scale, const float* dshift, const float* y, cudaStream_t s,
                      const unsigned char* mk, unsigned int* counter, const int32_t* order) {
  auto run = [&](auto kern) -> int {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    const int64_t need = (rows + kDynRows * 8 - 1) / (kDynRows * 8);  // blocks that can get a chunk
    int64_t grid = (int64_t)per_sm * sm_count();
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned int), s) != cudaSuccess) return SG_ERR_CUDA;
    kern<<<(unsigned)grid, 256, 0, s>>>(rows, ptr, idx, val, in, out, scale, dshift, y, mk, counter, order);
    return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
  };
  if (val) {
    if (dshift) return run(spmm_kernel<float, B, true, true, VAR, true>);
    return run(spmm_kernel<float, B, true, false, VAR, true>);
  }
  if (dshift) return run(spmm_kernel<float, B, false, true, VAR, true>);
  return run(spmm_kernel<float, B, false, false, VAR, true>);
}

template <int B>
int launch_spmm_dyn_b(int variant, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
                      const float* in, float* out, const float* scale, const float* dshift, const float* y,
                      cudaStream_t s, const unsigned char* mk, unsigned int* counter, const int32_t* order) {
  switch (variant) {
    case 0: return launch_spmm_dyn_v<B, 0>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 1: return launch_spmm_dyn_v<B, 1>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 2: return launch_spmm_dyn_v<B, 2>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 3: return launch_spmm_dyn_v<B, 3>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 4: return launch_spmm_dyn_v<B, 4>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 5: return launch_spmm_dyn_v<B, 5>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 6: return launch_spmm_dyn_v<B, 6>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    case 7: return launch_spmm_dyn_v<B, 7>(rows, ptr, idx, val, in, out, scale, dshift, y, s, mk, counter, order);
    default: return SG_ERR_ARG;
  }
}

__global__ void count_minmax(int64_t m, const double* __restrict__ cnt, unsigned long long* mm) {
  unsigned long long lo = ~0ull, hi = 0;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long c = (unsigned long long)cnt[j];
    lo = c < lo ? c : lo;
    hi = c > hi ? c : hi;
  }
  for (int o = 16; o; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, lo, o), b = __shfl_xor_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mm, lo);
    atomicMax(mm + 1, hi);
  }
}

// idf_kernel's rules from per-column cell counts instead of CSC column pointers
__global__ void idf_from_counts(int64_t n, int64_t m, const double* __restrict__ cnt,
                                const unsigned long long* __restrict__ mm, double* __restrict__ w) {
  const bool equal = mm[0] == mm[1];
  const double dn = (double)n;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    if (equal) { w[j] = 1.0; continue; }
    double c = cnt[j];
    if (c == 0.0) c = 1.0;
    else if (c == dn) c = dn - 1.0;
    w[j] = log(dn / c);
  }
}

__global__ void init_mm(unsigned long long* mm) { mm[0] = ~0ull; mm[1] = 0; }

extern "C" int sg_idf_from_counts(int64_t n, int64_t m, const double* counts, double* w, unsigned long long* mm,
                                  void* stream) {
  if (n < 1 || m < 0 || (m > 0 && (!counts || !w || !mm))) return SG_ERR_ARG;
  if (m == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  const int g = grid_for(m, 256, 4 * sm_count());
  init_mm<<<1, 1, 0, s>>>(mm);
  count_minmax<<<g, 256, 0, s>>>(m, counts, mm);
  idf_from_counts<<<g, 256, 0, s>>>(n, m, counts, mm, w);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_csr_row_norms(int64_t n, const int64_t* indptr, const int32_t* indices, const float* values,
                                const double* w, double* rinv, int* status, unsigned long long* bad, void* stream) {
  if (n < 0 || (n > 0 && (!indptr || !w || !rinv || !status))) return SG_ERR_ARG;
  if (n == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  rownorm_kernel<<<grid_for(n * 32, 256, 8 * sm_count()), 256, 0, s>>>(n, indptr, indices, values, w, rinv, status,
                                                                      bad);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_spmm_variants(void) { return kSpmmVariants; }

namespace sg {
namespace {
int spmm_dyn_impl(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
                  const void* in, void* out, const void* scale, const void* dshift, const void* y, int variant,
                  const int32_t* order, const unsigned char* row_mask, unsigned int* counter, void* stream) {
  if (rows < 0 || rows >= (int64_t(1) << 31) || !scale || (dshift && !y) || !counter || variant < 0 ||
      variant >= kSpmmVariants || dtype != 0)
    return SG_ERR_ARG;
  if (rows == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  const float *fi = (const float*)in, *fs = (const float*)scale, *fd = (const float*)dshift, *fy = (const float*)y;
  float* fo = (float*)out;
  switch (block) {
    case 4: return launch_spmm_dyn_b<4>(variant, rows, ptr, idx, val, fi, fo, fs, fd, fy, s, row_mask, counter, order);
    case 8: return launch_spmm_dyn_b<8>(variant, rows, ptr, idx, val, fi, fo, fs, fd, fy, s, row_mask, counter, order);
    case 16:
      return launch_spmm_dyn_b<16>(variant, rows, ptr, idx, val, fi, fo, fs, fd, fy, s, row_mask, counter, order);
    case 32:
      return launch_spmm_dyn_b<32>(variant, rows, ptr, idx, val, fi, fo, fs, fd, fy, s, row_mask, counter, order);
    default: return SG_ERR_ARG;
  }
}

// keys: ~len (descending length under an ascending sort), values: row index
__global__ void order_keys_kernel(int64_t rows, const int64_t* __restrict__ ptr, uint64_t* __restrict__ keys,
                                  uint64_t* __restrict__ vals) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < rows; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t len = ptr[r + 1] - ptr[r];
    keys[r] = 0xffffffffull - (uint64_t)(len < 0xffffffffll ? len : 0xffffffffll);
    vals[r] = (uint64_t)r;
  }
}

// position p = 4c + j holds the row of sorted rank c + j·C (C = ceil(rows/4)):
// each 4-row fetch gets one row of every quarter of the length order
__global__ void order_deal_kernel(int64_t rows, int64_t C, const uint64_t* __restrict__ sorted_rows,
                                  int32_t* __restrict__ order) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < 4 * C; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = p >> 2, j = p & 3;
    const int64_t q = c + j * C;
    order[p] = q < rows ? (int32_t)sorted_rows[q] : -1;
  }
}

struct OrderLayout {
  uint64_t *keys, *vals, *keys_alt, *vals_alt;
  void* radix;
  int64_t bytes;
};

OrderLayout order_layout(char* base, int64_t rows) {
  OrderLayout L{};
  int64_t o = 0;
  auto take = [&](int64_t b) { const int64_t r = o; o += (b + 255) / 256 * 256; return r; };
  const int64_t R = rows > 0 ? rows : 1;
  const int64_t ok = take(8 * R), ov = take(8 * R), oka = take(8 * R), ova = take(8 * R), orad = take(radix_scratch_bytes(R));
  if (base) {
    L.keys = (uint64_t*)(base + ok);
    L.vals = (uint64_t*)(base + ov);
    L.keys_alt = (uint64_t*)(base + oka);
    L.vals_alt = (uint64_t*)(base + ova);
    L.radix = base + orad;
  }
  L.bytes = o;
  return L;
}
}  // namespace
}  // namespace sg

extern "C" int sg_spmm_dyn(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx,
                           const float* val, const void* in, void* out, const void* scale, const void* dshift,
                           const void* y, int variant, const unsigned char* row_mask, unsigned int* counter,
                           void* stream) {
  return spmm_dyn_impl(dtype, block, rows, ptr, idx, val, in, out, scale, dshift, y, variant, nullptr, row_mask,
                       counter, stream);
}

extern "C" int sg_spmm_dyn_ordered(int dtype, int block, int64_t positions, const int64_t* ptr, const int32_t* idx,
                                   const float* val, const void* in, void* out, const void* scale,
                                   const void* dshift, const void* y, int variant, const int32_t* order,
                                   unsigned int* counter, void* stream) {
  if (!order) return SG_ERR_ARG;
  return spmm_dyn_impl(dtype, block, positions, ptr, idx, val, in, out, scale, dshift, y, variant, order, nullptr,
                       counter, stream);
}

extern "C" int64_t sg_row_order_positions(int64_t rows) { return rows < 0 ? -1 : 4 * ((rows + 3) / 4); }

extern "C" int64_t sg_row_order_scratch_bytes(int64_t rows) { return rows < 0 ? -1 : order_layout(nullptr, rows).bytes; }

extern "C" int sg_row_order(int64_t rows, const int64_t* ptr, int32_t* order, void* scratch, int64_t scratch_bytes,
                            void* stream) {
  if (rows < 0 || rows >= (int64_t(1) << 31) || (rows > 0 && (!ptr || !order || !scratch))) return SG_ERR_ARG;
  if (((uintptr_t)scratch & 255u) != 0) return SG_ERR_ARG;
  if (rows == 0) return SG_OK;
  OrderLayout L = order_layout((char*)scratch, rows);
  if (scratch_bytes < L.bytes) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  const int g = grid_for(rows, 256, 16 * sm_count());
  order_keys_kernel<<<g, 256, 0, s>>>(rows, ptr, L.keys, L.vals);
  SG_CHECK_LAUNCH();
  bool alt = false;
  if (radix_sort_u64(rows, L.keys, L.vals, L.keys_alt, L.vals_alt, 0, 32, L.radix, s, &alt) != cudaSuccess)
    return SG_ERR_CUDA;
  const int64_t C = (rows + 3) / 4;
  order_deal_kernel<<<grid_for(4 * C, 256, 16 * sm_count()), 256, 0, s>>>(rows, C, alt ? L.vals_alt : L.vals, order);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_spmm_masked(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx,
                              const float* val, const void* in, void* out, const void* scale, const void* dshift,
                              const void* y, int grid, int variant, const unsigned char* row_mask, void* stream) {
  if (rows < 0 || !scale || (dshift && !y) || variant < 0 || variant >= kSpmmVariants) return SG_ERR_ARG;
  if (rows == 0) return SG_OK;
  if (grid <= 0) grid = grid_for(rows * 32, 256, 8 * sm_count() * 4);
  cudaStream_t s = as_stream(stream);
  if (dtype == 0)
    return launch_spmm<float>(variant, block, rows, ptr, idx, val, (const float*)in, (float*)out,
                              (const float*)scale, (const float*)dshift, (const float*)y, grid, s, row_mask);
  if (dtype == 1)
    return launch_spmm<double>(variant, block, rows, ptr, idx, val, (const double*)in, (double*)out,
                               (const double*)scale, (const double*)dshift, (const double*)y, grid, s, row_mask);
  return SG_ERR_ARG;
}

extern "C" int sg_spmm_ex(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx,
                          const float* val, const void* in, void* out, const void* scale, const void* dshift,
                          const void* y, int grid, int variant, void* stream) {
  return sg_spmm_masked(dtype, block, rows, ptr, idx, val, in, out, scale, dshift, y, grid, variant, nullptr, stream);
}

extern "C" int sg_spmm(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx,
                       const float* val, const void* in, void* out, const void* scale, const void* dshift,
                       const void* y, int grid, void* stream) {
  return sg_spmm_ex(dtype, block, rows, ptr, idx, val, in, out, scale, dshift, y, grid, 0, stream);
}
