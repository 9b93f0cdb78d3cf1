// Compensated FP32 SpMM for the eigensolver's FP64 correction sweep.
//
// The sweep applies the Gram operator A v = a ⊙ X (w² ⊙ Xᵀ (a ⊙ v)) − D⁻¹ v
// (snapatac2-python/src/embedding.rs:133-152) to the k <= 32 Ritz vectors
// once, in FP64-class precision.  On GB300 FP64 runs at 1/64 of the FP32
// rate, and an FP64 SpMM over 32 columns is bound by its additions, not by its
// gathers.  Here every FP64 operand value v is stored as an FP32 pair
// (hi, lo), hi = fl32(v), lo = fl32(v − hi), so hi + lo equals v to within
// 2^-48 |v|.  Each output is carried as an FP32 sum s and an FP32
// compensation c.  s is updated by Knuth's TwoSum (The Art of Computer
// Programming, vol. 2, 4.2.2), which recovers the rounding error of every
// addition exactly; the errors and the lo parts accumulate in c.  With k terms
// the sum s + c is within about k·2^-48 of Σ|terms| — FP64-class — at FP32
// instruction rates.  With valued X (FP32 values x) each product x·hi is
// split exactly by an FMA (p = x·hi, fma(x, hi, −p) = its rounding error).
//
// Layout: 32 columns per row, each (hi, lo), so a row is 256 bytes, 16
// float4 vectors; 16 lanes per nonzero, 2 nonzeros per warp step, as the FP64
// form of the gather kernel (csrc/spectral.cu).  The partial sums of the two
// half-warps are combined by one TwoSum: a fixed order, deterministic.
//   pass 0 (Xᵀ pass): out[r] = pairs of scale[r] · Σ x_e in[col_e]
//   pass 1 (X pass):  out[r] = scale[r] · Σ x_e in[col_e] − dshift[r] · y[r]  (FP64)
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kDsCols = 32;
constexpr int kDsVec = kDsCols / 2;  // float4 vectors per row: two columns each
constexpr int kDsRows = 4;           // rows a warp takes per counter fetch (dynamic schedule)

__device__ __forceinline__ void two_sum_acc(float& s, float& c, float x) {
  const float t = s + x;
  const float z = t - s;
  c += (s - (t - z)) + (x - z);
  s = t;
}

template <bool VALUED, bool XPASS, int CH, bool DYN>
__global__ void __launch_bounds__(256)
spmm_ds_kernel(int64_t rows, const int64_t* __restrict__ ptr, const int32_t* __restrict__ idx,
               const float* __restrict__ val, const float4* __restrict__ in, void* __restrict__ out,
               const double* __restrict__ scale, const double* __restrict__ dshift, const double* __restrict__ y,
               unsigned int* __restrict__ counter, const int32_t* __restrict__ order) {
  constexpr int LPN = kDsVec, NPS = 32 / LPN;
  const int lane = threadIdx.x & 31;
  const int sub = lane % LPN, slot = lane / LPN;
  const int64_t gw = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  int64_t r = DYN ? 0 : gw, rend = DYN ? 0 : rows;
  while (true) {
    if (DYN) {
      if (r >= rend) {
        unsigned int c0 = 0;
        if (lane == 0) c0 = atomicAdd(counter, (unsigned int)kDsRows);
        c0 = __shfl_sync(0xffffffffu, c0, 0);
        r = c0;
        rend = r + kDsRows < rows ? r + kDsRows : rows;
        if (r >= rows) break;
      }
    } else if (r >= rows) {
      break;
    }
    int64_t rr = r;
    r += DYN ? 1 : nw;
    if (DYN && order) {  // position -> row (-1: none), longest rows first
      rr = order[rr];
      if (rr < 0) continue;
    }
    const int64_t s = ptr[rr], e = ptr[rr + 1];
    float s0 = 0.f, c0 = 0.f, s1 = 0.f, c1 = 0.f;
    for (int64_t base = s; base < e; base += 32 * CH) {
      int ci[CH];
      float cv[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const int64_t k = base + c * 32 + lane;
        ci[c] = k < e ? __ldg(idx + k) : -1;
        cv[c] = (VALUED && k < e) ? __ldg(val + k) : 1.0f;
      }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        float4 g[LPN];
        float gv[LPN];
#pragma unroll
        for (int j = 0; j < LPN; ++j) {
          const int col = __shfl_sync(0xffffffffu, ci[c], j * NPS + slot);
          if (VALUED) gv[j] = __shfl_sync(0xffffffffu, cv[c], j * NPS + slot);
          g[j] = col >= 0 ? __ldg(in + (int64_t)col * kDsVec + sub) : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int j = 0; j < LPN; ++j) {
          if (VALUED) {
            const float x = gv[j];
            const float p0 = x * g[j].x, p1 = x * g[j].z;
            const float e0 = fmaf(x, g[j].x, -p0), e1 = fmaf(x, g[j].z, -p1);
            two_sum_acc(s0, c0, p0);
            two_sum_acc(s1, c1, p1);
            c0 += fmaf(x, g[j].y, e0);
            c1 += fmaf(x, g[j].w, e1);
          } else {
            two_sum_acc(s0, c0, g[j].x);
            two_sum_acc(s1, c1, g[j].z);
            c0 += g[j].y;
            c1 += g[j].w;
          }
        }
      }
    }
    // the two half-warps' sums: s + s' by TwoSum, compensations added
#pragma unroll
    for (int o = LPN; o < 32; o <<= 1) {
      const float t0 = __shfl_xor_sync(0xffffffffu, s0, o), u0 = __shfl_xor_sync(0xffffffffu, c0, o);
      const float t1 = __shfl_xor_sync(0xffffffffu, s1, o), u1 = __shfl_xor_sync(0xffffffffu, c1, o);
      c0 += u0;
      c1 += u1;
      two_sum_acc(s0, c0, t0);
      two_sum_acc(s1, c1, t1);
    }
    if (slot == 0) {
      const double sc = scale[rr];
      const double v0 = sc * ((double)s0 + (double)c0), v1 = sc * ((double)s1 + (double)c1);
      if (XPASS) {
        double2 o;
        if (dshift) {
          const double d = dshift[rr];
          const double2 yy = *reinterpret_cast<const double2*>(y + rr * kDsCols + 2 * sub);
          o.x = v0 - d * yy.x;
          o.y = v1 - d * yy.y;
        } else {
          o.x = v0;
          o.y = v1;
        }
        *reinterpret_cast<double2*>(static_cast<double*>(out) + rr * kDsCols + 2 * sub) = o;
      } else {
        const float h0 = (float)v0, h1 = (float)v1;
        static_cast<float4*>(out)[rr * kDsVec + sub] =
            make_float4(h0, (float)(v0 - (double)h0), h1, (float)(v1 - (double)h1));
      }
    }
  }
}

// out[r, c] = pairs of a[r] · U[r, c] (a NULL: of U), U n x 32 FP64
__global__ void ds_split_kernel(int64_t n, const double* __restrict__ a, const double* __restrict__ U,
                                float2* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * kDsCols;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double v = a ? a[t / kDsCols] * U[t] : U[t];
    const float h = (float)v;
    out[t] = make_float2(h, (float)(v - (double)h));
  }
}

int sm_count_ds() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

template <bool VALUED, bool XPASS, int CH, bool DYN>
int launch_ds(int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val, const void* in, void* out,
              const double* scale, const double* dshift, const double* y, unsigned int* counter,
              const int32_t* order, cudaStream_t s) {
  auto kern = spmm_ds_kernel<VALUED, XPASS, CH, DYN>;
  int64_t grid;
  if (DYN) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0) != cudaSuccess || per_sm < 1)
      per_sm = 1;
    const int64_t need = (rows + kDsRows * 8 - 1) / (kDsRows * 8);
    grid = (int64_t)per_sm * sm_count_ds();
    if (grid > need) grid = need;
    if (grid < 1) grid = 1;
    if (cudaMemsetAsync(counter, 0, sizeof(unsigned int), s) != cudaSuccess) return SG_ERR_CUDA;
  } else {
    grid = grid_for(rows * 32, 256, 32 * sm_count_ds());
  }
  kern<<<(unsigned)grid, 256, 0, s>>>(rows, ptr, idx, val, static_cast<const float4*>(in), out, scale, dshift, y,
                                      counter, order);
  return cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

template <bool VALUED, bool XPASS>
int launch_ds_v(int variant, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val, const void* in,
                void* out, const double* scale, const double* dshift, const double* y, unsigned int* counter,
                const int32_t* order, cudaStream_t s) {
  switch (variant) {
    case 0: return launch_ds<VALUED, XPASS, 1, false>(rows, ptr, idx, val, in, out, scale, dshift, y, counter, nullptr, s);
    case 1: return launch_ds<VALUED, XPASS, 2, false>(rows, ptr, idx, val, in, out, scale, dshift, y, counter, nullptr, s);
    case 2: return launch_ds<VALUED, XPASS, 1, true>(rows, ptr, idx, val, in, out, scale, dshift, y, counter, order, s);
    case 3: return launch_ds<VALUED, XPASS, 2, true>(rows, ptr, idx, val, in, out, scale, dshift, y, counter, order, s);
    default: return SG_ERR_ARG;
  }
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_spmm_ds_variants(void) { return 4; }

extern "C" int sg_spmm_ds(int pass, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
                          const void* in, void* out, const double* scale, const double* dshift, const double* y,
                          int variant, const int32_t* order, unsigned int* counter, void* stream) {
  if ((pass != 0 && pass != 1) || rows < 0 || rows >= (int64_t(1) << 31) || variant < 0 || variant > 3 ||
      (rows > 0 && (!ptr || !idx || !in || !out || !scale)) || (dshift && (!y || pass == 0)) ||
      (variant >= 2 && !counter) || (order && variant < 2))
    return SG_ERR_ARG;
  if (((uintptr_t)in & 15u) != 0 || ((uintptr_t)out & 15u) != 0 || (y && ((uintptr_t)y & 15u) != 0))
    return SG_ERR_ARG;
  if (rows == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  if (val) {
    if (pass) return launch_ds_v<true, true>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, counter, order, s);
    return launch_ds_v<true, false>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, counter, order, s);
  }
  if (pass) return launch_ds_v<false, true>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, counter, order, s);
  return launch_ds_v<false, false>(variant, rows, ptr, idx, val, in, out, scale, dshift, y, counter, order, s);
}

extern "C" int sg_ds_split(int64_t n, const double* a, const double* U, void* out, void* stream) {
  if (n < 0 || (n > 0 && (!U || !out))) return SG_ERR_ARG;
  if (n == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  ds_split_kernel<<<grid_for(n * kDsCols, 256, 16 * sm_count_ds()), 256, 0, s>>>(n, a, U,
                                                                                   static_cast<float2*>(out));
  SG_CHECK_LAUNCH();
  return SG_OK;
}
