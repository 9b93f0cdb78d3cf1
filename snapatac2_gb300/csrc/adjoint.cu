// Adjoint of the matrix-free cosine spectral operator: gradient of the sum of
// the wanted eigenvalues with respect to the per-feature weights w.
//
// Forward chain (as in snapatac2-python/src/embedding.rs:139-152,315-326 with
// user feature weights): r_i = 1/||(XW)_i||, Xn = R X W, c = Xnᵀ1, d = Xn c,
// s = (d - 1)^(-1/2), A = S (Xn Xnᵀ - I) S, f = sum_l λ_l over the wanted
// eigenpairs (A U = U Λ).  Reverse mode (∂f/∂A = U Uᵀ):
//   q_i  = sum_l λ_l U_il²,   δ̄_i = -q_i s_i²,  V = S U
//   [Z | e | h] = Xᵀ [r⊙V | r⊙δ̄ | r]                        (CSC SpMM)
//   [P1 | P2]   = X  [w²⊙Z | w²⊙e]                          (CSR SpMM)
//   ρ̄_i = -r_i (2 V_i·(r_i P1_i) + δ̄_i d_i + r_i P2_i)
//   g    = (X∘X)ᵀ (ρ̄ ⊙ r)                                   (CSC SpMM)
//   ∂f/∂w_j = w_j (2 ||Z_j||² + 2 h_j e_j + g_j)
// The three SpMMs use sg_spmm(_ex) in FP64; this file holds the elementwise
// stages between them.  Everything is FP64.
#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

// out (n x B): [r s U | r δ̄ | r | 0...];  dbar = δ̄
__global__ void stage1_kernel(int64_t n, int k, const double* __restrict__ U, const double* __restrict__ lam,
                              const double* __restrict__ dinv, const double* __restrict__ rinv, int B,
                              double* __restrict__ out, double* __restrict__ dbar) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double s = sqrt(dinv[i]), r = rinv[i];
    double q = 0.0;
    for (int l = 0; l < k; ++l) {
      const double u = U[i * k + l];
      q = fma(lam[l] * u, u, q);
      out[i * B + l] = r * s * u;
    }
    const double db = -q * s * s;
    dbar[i] = db;
    out[i * B + k] = r * db;
    out[i * B + k + 1] = r;
    for (int c = k + 2; c < B; ++c) out[i * B + c] = 0.0;
  }
}

// out (m x B2): [w² Z | w² e | 0...] from ZEH = [Z | e | h] (m x B)
__global__ void stage2_kernel(int64_t m, int k, const double* __restrict__ zeh, int B, const double* __restrict__ w,
                              int B2, double* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    const double w2 = w[j] * w[j];
    for (int l = 0; l <= k; ++l) out[j * B2 + l] = w2 * zeh[j * B + l];
    for (int c = k + 1; c < B2; ++c) out[j * B2 + c] = 0.0;
  }
}

// out (n x 4): [ρ̄ ⊙ r, 0, 0, 0] from P = [P1 | P2] (n x B2)
__global__ void stage3_kernel(int64_t n, int k, const double* __restrict__ U, const double* __restrict__ dinv,
                              const double* __restrict__ rinv, const double* __restrict__ dbar,
                              const double* __restrict__ P, int B2, double* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double s = sqrt(dinv[i]), r = rinv[i];
    const double d = 1.0 / dinv[i] + 1.0;
    double vp = 0.0;
    for (int l = 0; l < k; ++l) vp = fma(s * U[i * k + l], r * P[i * B2 + l], vp);
    const double t = 2.0 * vp + dbar[i] * d + r * P[i * B2 + k];
    const double rho_bar = -r * t;
    out[i * 4 + 0] = rho_bar * r;
    out[i * 4 + 1] = 0.0;
    out[i * 4 + 2] = 0.0;
    out[i * 4 + 3] = 0.0;
  }
}

__global__ void final_kernel(int64_t m, int k, const double* __restrict__ w, const double* __restrict__ zeh, int B,
                             const double* __restrict__ g, double* __restrict__ grad) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
    double zz = 0.0;
    for (int l = 0; l < k; ++l) zz = fma(zeh[j * B + l], zeh[j * B + l], zz);
    const double e = zeh[j * B + k], h = zeh[j * B + k + 1];
    grad[j] = w[j] * (2.0 * zz + 2.0 * h * e + g[j * 4]);
  }
}

__global__ void square_kernel(int64_t n, const float* __restrict__ in, float* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    out[t] = in[t] * in[t];
}

int sms() {
  int dev = 0, s = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
  return s > 0 ? s : 1;
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int sg_adjoint_stage1(int64_t n, int k, const double* U, const double* evals, const double* dinv,
                                 const double* rinv, int block, double* out, double* dbar, void* stream) {
  if (n <= 0 || k <= 0 || block < k + 2) return SG_ERR_ARG;
  stage1_kernel<<<grid_for(n, 256, 16 * sms()), 256, 0, as_stream(stream)>>>(n, k, U, evals, dinv, rinv, block, out,
                                                                              dbar);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_adjoint_stage2(int64_t m, int k, const double* zeh, int block, const double* w, int block2,
                                 double* out, void* stream) {
  if (m <= 0 || k <= 0 || block < k + 2 || block2 < k + 1) return SG_ERR_ARG;
  stage2_kernel<<<grid_for(m, 256, 16 * sms()), 256, 0, as_stream(stream)>>>(m, k, zeh, block, w, block2, out);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_adjoint_stage3(int64_t n, int k, const double* U, const double* dinv, const double* rinv,
                                 const double* dbar, const double* P, int block2, double* out, void* stream) {
  if (n <= 0 || k <= 0 || block2 < k + 1) return SG_ERR_ARG;
  stage3_kernel<<<grid_for(n, 256, 16 * sms()), 256, 0, as_stream(stream)>>>(n, k, U, dinv, rinv, dbar, P, block2,
                                                                              out);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_adjoint_final(int64_t m, int k, const double* w, const double* zeh, int block, const double* g,
                                double* grad, void* stream) {
  if (m <= 0 || k <= 0 || block < k + 2) return SG_ERR_ARG;
  final_kernel<<<grid_for(m, 256, 16 * sms()), 256, 0, as_stream(stream)>>>(m, k, w, zeh, block, g, grad);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int sg_square_values(int64_t nnz, const float* values, float* out, void* stream) {
  if (nnz < 0) return SG_ERR_ARG;
  if (nnz == 0) return SG_OK;
  square_kernel<<<grid_for(nnz, 256, 16 * sms()), 256, 0, as_stream(stream)>>>(nnz, values, out);
  SG_CHECK_LAUNCH();
  return SG_OK;
}
