// One-call eigensolver of the cosine operator: thick-restart block Lanczos
// (Krylov-Schur) with full reorthogonalisation, replacing the ARPACK call of
// the reference's eigen (snapatac2-python/src/embedding.rs:155-188:
// eigsh(LinearOperator(f), k, v0, which='LM'), sorted descending).
//
// The host loop runs here: block expansions (two SpMM launches, two passes of
// classical Gram-Schmidt, two Cholesky-QR passes, the block of H), and when
// the basis is full the Rayleigh-Ritz step on the GPU in FP64 (ritz.cu), the
// selection of the kept Ritz pairs, the residual test and the restart
// Q <- Q Y_keep -- all on the device.  The host reads one small decision
// record per restart (and the solve's last one); nothing else crosses PCIe.
//
// precision 0 ("mixed"): X pattern, basis, SpMM in FP32 with FP32
// accumulation (cross-CTA sums in FP64); H, Ritz problem, output vectors FP64;
// an optional final FP64 correction sweep (one FP64 block matvec of the Ritz
// vectors and a Rayleigh-Ritz on their span).  precision 1: all FP64.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace sg {
namespace {

constexpr int kStaged = 100;
constexpr int kDyn = 200;
constexpr double kFp32Floor = 3e-5;  // residual level (x |A|) of a stalled FP32 solve

// ---------------------------------------------------------------------------
// Order of the nw candidate Ritz values by |θ| descending, ties by ascending
// value (numpy's stable argsort of -|θ| over eigh's ascending output):
// ord[pos] = candidate.  The keep first ones, as ascending candidate indices,
// go to sel, with their rows in the eigenvector array in row_of (-1 for the
// others): only those get eigenvectors (the candidates' dense bulk would
// chain into long clusters for inverse iteration).  One CTA.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(512)
order_kernel(int nw, const double* __restrict__ lam, int keep, int* __restrict__ ord, int* __restrict__ sel,
             int* __restrict__ row_of) {
  extern __shared__ int spos[];  // nw
  for (int c = threadIdx.x; c < nw; c += blockDim.x) {
    const double ac = fabs(lam[c]);
    int pos = 0;
    for (int o = 0; o < nw; ++o) {
      const double ao = fabs(lam[o]);
      pos += (ao > ac) || (ao == ac && o < c);
    }
    ord[pos] = c;
    spos[c] = pos;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int j = 0;
    for (int c = 0; c < nw; ++c) {
      if (spos[c] < keep) {
        sel[j] = c;
        row_of[c] = j++;
      } else {
        row_of[c] = -1;
      }
    }
  }
}

// Ritz selection (one CTA).  Writes
//   ctl[0] worst residual / bar over the wanted k, ctl[1] largest residual,
//   ctl[2] max |θ|, ctl[3] status word, ctl[4..7] next Ritz values (NaN)
//   theta_keep, Yk (Me x keep): kept pairs for the restart
//   Bc (b x keep) = Rl Yk[Me-b:Me, :], Rl = H[Me:Me+b, Me-b:Me]
//   Yf (Me x k), evals_f, res_f: wanted pairs sorted by θ descending
__global__ void __launch_bounds__(512)
select_kernel(int Me, int nw, const double* __restrict__ lam, const int* __restrict__ ord,
              const int* __restrict__ row_of, const double* __restrict__ Zt, const double* __restrict__ H, int64_t ldh,
              int b, int k, int keep, double tol_vec, double tol_val, int vpos, const int* __restrict__ status,
              double* __restrict__ ctl, double* __restrict__ theta_keep, double* __restrict__ Yk,
              double* __restrict__ Bc, double* __restrict__ Yf, double* __restrict__ evals_f,
              double* __restrict__ res_f) {
  extern __shared__ double ssel[];
  double* res = ssel;                                // k
  int* fpos = reinterpret_cast<int*>(ssel + k);      // k
  auto vec = [&](int c) { return Zt + (size_t)row_of[ord[c]] * Me; };  // c < keep
  const double* Rl = H + (int64_t)Me * ldh + (Me - b);
  for (int s = threadIdx.x; s < k; s += blockDim.x) {
    const double* y = vec(s) + (Me - b);
    double r2 = 0.0;
    for (int r = 0; r < b; ++r) {
      double t = 0.0;
      for (int q = 0; q < b; ++q) t = fma(Rl[(int64_t)r * ldh + q], y[q], t);
      r2 = fma(t, t, r2);
    }
    res[s] = sqrt(r2);
    // final position: θ descending, ties in Ritz order
    const double th = lam[ord[s]];
    int fp = 0;
    for (int o = 0; o < k; ++o) {
      const double to = lam[ord[o]];
      fp += (to > th) || (to == th && o < s);
    }
    fpos[s] = fp;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < Me * keep; t += blockDim.x) {
    const int p = t / keep, c = t % keep;
    Yk[t] = vec(c)[p];
  }
  for (int c = threadIdx.x; c < keep; c += blockDim.x) theta_keep[c] = lam[ord[c]];
  for (int t = threadIdx.x; t < b * keep; t += blockDim.x) {
    const int r = t / keep, c = t % keep;
    const double* y = vec(c) + (Me - b);
    double s = 0.0;
    for (int q = 0; q < b; ++q) s = fma(Rl[(int64_t)r * ldh + q], y[q], s);
    Bc[t] = s;
  }
  for (int t = threadIdx.x; t < Me * k; t += blockDim.x) {
    const int p = t / k, s = t % k;
    Yf[(size_t)p * k + fpos[s]] = vec(s)[p];
  }
  for (int s = threadIdx.x; s < k; s += blockDim.x) {
    evals_f[fpos[s]] = lam[ord[s]];
    res_f[fpos[s]] = res[s];
  }
  if (threadIdx.x == 0) {
    const double anorm = fmax(fmax(fabs(lam[0]), fabs(lam[nw - 1])), 1e-300);
    double worst = 0.0, hist = 0.0;
    for (int s = 0; s < k; ++s) {
      const double th = lam[ord[s]];
      const double bar = ((th > 0.0) || !vpos ? tol_vec : tol_val) * anorm;
      worst = fmax(worst, res[s] / bar);
      hist = fmax(hist, res[s]);
    }
    ctl[0] = worst;
    ctl[1] = hist;
    ctl[2] = anorm;
    ctl[3] = (double)*status;
    for (int q = 0; q < 4; ++q)
      ctl[4 + q] = k + q < nw ? lam[ord[k + q]] : __longlong_as_double(0x7ff8000000000000ll);
  }
}

// Restarted H: diag(θ_keep), coupling Bc below the kept block and its transpose.
__global__ void hrestart_kernel(double* __restrict__ H, int64_t ldh, int ld, int keep, int b,
                                const double* __restrict__ theta_keep, const double* __restrict__ Bc) {
  const int64_t tot = (int64_t)ld * ld;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot; t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / ld), j = (int)(t % ld);
    double v = 0.0;
    if (i == j && i < keep) v = theta_keep[i];
    else if (i >= keep && i < keep + b && j < keep) v = Bc[(int64_t)(i - keep) * keep + j];
    else if (j >= keep && j < keep + b && i < keep) v = Bc[(int64_t)(j - keep) * keep + i];
    H[(int64_t)i * ldh + j] = v;
  }
}

// Final correction sweep, small part (one CTA): G = RᵀR (Cholesky of the
// symmetrised k x k Gram matrix), Ri = R⁻¹, C = Riᵀ sym(Hm) Ri.
__global__ void refine_prep_kernel(int k, int kb, const double* __restrict__ G, const double* __restrict__ Hm,
                                   double* __restrict__ Ri, double* __restrict__ C, double* __restrict__ tmp,
                                   int* __restrict__ status) {
  __shared__ double R[32][33];
  __shared__ double I[32][33];
  __shared__ int bad;
  if (threadIdx.x == 0) {
    bad = 0;
    for (int j = 0; j < k && !bad; ++j) {
      for (int c = j; c < k; ++c) {
        double s = 0.5 * (G[j * kb + c] + G[c * kb + j]);
        for (int i = 0; i < j; ++i) s -= R[i][j] * R[i][c];
        if (c == j) {
          if (!(s > 0.0)) { bad = 1; break; }
          R[j][j] = sqrt(s);
        } else {
          R[j][c] = s / R[j][j];
        }
      }
      for (int c = 0; c < j; ++c) R[j][c] = 0.0;
    }
    if (!bad) {  // inverse of the upper triangular R, column by column
      for (int c = 0; c < k; ++c) {
        for (int r = k - 1; r >= 0; --r) {
          double s = r == c ? 1.0 : 0.0;
          for (int q = r + 1; q < k; ++q) s -= R[r][q] * I[q][c];
          I[r][c] = s / R[r][r];
        }
      }
    } else {
      atomicCAS(status, 0, SG_ERR_NUMERIC);
    }
  }
  __syncthreads();
  if (bad) return;
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) Ri[t] = I[t / k][t % k];
  // tmp = sym(Hm) Ri, C = Riᵀ tmp
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
    const int r = t / k, c = t % k;
    double s = 0.0;
    for (int q = 0; q < k; ++q) s = fma(0.5 * (Hm[r * kb + q] + Hm[q * kb + r]), I[q][c], s);
    tmp[t] = s;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < k * k; t += blockDim.x) {
    const int r = t / k, c = t % k;
    double s = 0.0;
    for (int q = 0; q < k; ++q) s = fma(I[q][r], tmp[q * k + c], s);
    C[t] = s;
  }
}

// Of the kr refined pairs (lam ascending, Z rows = eigenvectors of C) the k
// of largest |λ| (ties: the smaller value first, as numpy's stable argsort of
// -|θ| over eigh's ascending output), in descending eigenvalue order:
// Y = Ri Z[:, chosen] (kr x k), evals descending.  One CTA.
__global__ void refine_finish_kernel(int k, int kr, const double* __restrict__ Ri, const double* __restrict__ lam,
                                     const double* __restrict__ Zt, double* __restrict__ Y,
                                     double* __restrict__ evals) {
  __shared__ int pick[32];
  if (threadIdx.x == 0) {
    int c = 0;
    for (int i = kr - 1; i >= 0; --i) {  // descending value
      const double ai = fabs(lam[i]);
      int pos = 0;
      for (int o = 0; o < kr; ++o) {
        const double ao = fabs(lam[o]);
        pos += (ao > ai) || (ao == ai && o < i);
      }
      if (pos < k) pick[c++] = i;
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kr * k; t += blockDim.x) {
    const int p = t / k, c = t % k;
    const double* z = Zt + (size_t)pick[c] * kr;
    double s = 0.0;
    for (int q = 0; q < kr; ++q) s = fma(Ri[p * kr + q], z[q], s);
    Y[t] = s;
  }
  for (int c = threadIdx.x; c < k; c += blockDim.x) evals[c] = lam[pick[c]];
}

// ---------------------------------------------------------------------------
struct Basis {
  int M, keep;
};

// keep ≈ 3.2 k, M ≈ keep + max(18 blocks, 7.5 k), at most the Rayleigh-Ritz
// limit (k = 30: keep 96; M 320 at blocks 4 and 8, 384 at 16, 608 at 32).
// Measured at 100,000 cells x 500,000 features, block 16, residual bar 3e-9:
// keep 96 / M 384 took 132 block matvecs and 6 restarts (611 ms), keep 80 /
// M 320 140 and 8 (638 ms), keep 80 / M 256 148 and 12 (672 ms).
Basis default_basis(int k, int b) {
  int keep = std::max(k + 2 * b, (int)std::nearbyint(3.2 * k));
  int M = keep + std::max(18 * b, (int)std::nearbyint(7.5 * k));
  M = (M + b - 1) / b * b;
  M = std::min(M, (kRitzMaxN - b) / b * b);
  return {M, keep};
}

struct Work {
  char *Q, *Q2, *Z, *Zs, *W, *T;
  double *part, *C1, *C2, *G, *R1, *R2, *Rinv, *Rout, *H, *ctl, *theta_keep, *Yk, *Bc, *Yf, *evals_f, *res_f;
  int *ord, *sel, *row_of;
  unsigned* counter;
  RitzLayout ritz;
  // correction sweep
  double *Up, *Zs64, *W64, *T64, *part32, *G32, *H32, *Ri, *Cs, *tmp, *Yr, *ev32;
  RitzLayout ritz32;
  int64_t bytes;
};

Work layout(char* base, int code, int b, int k, int64_t n, int64_t m, int M, int nparts) {
  Work w{};
  int64_t o = 0;
  auto take = [&](int64_t bytes) { const int64_t r = o; o += (bytes + 255) / 256 * 256; return r; };
  const int64_t e = code ? 8 : 4;
  const int ld = M + b;
  const int64_t oQ = take(n * ld * e), oQ2 = take(n * ld * e), oZ = take(n * b * e), oZs = take(n * b * e),
                oW = take(n * b * e), oT = take(m * b * e), opart = take((int64_t)nparts * ld * b * 8),
                oC1 = take((int64_t)ld * b * 8), oC2 = take((int64_t)ld * b * 8), oG = take(b * b * 8),
                oR1 = take(b * b * 8), oR2 = take(b * b * 8), oRi = take(b * b * 8), oRo = take(b * b * 8),
                oH = take((int64_t)ld * ld * 8), octl = take(8 * 8), oth = take((int64_t)ld * 8),
                oYk = take((int64_t)ld * ld * 8), oBc = take((int64_t)b * ld * 8), oYf = take((int64_t)ld * k * 8),
                oef = take((int64_t)k * 8), orf = take((int64_t)k * 8), ocnt = take(2 * 4),
                oord = take((int64_t)ld * 4), osel = take((int64_t)ld * 4), orow = take((int64_t)ld * 4);
  const RitzLayout rl = ritz_layout(nullptr, M, M);
  const int64_t orl = take(rl.bytes);
  const bool refine = code == 0 && k <= 32;
  const int kb = 32;
  int64_t oUp = 0, oZs64 = 0, oW64 = 0, oT64 = 0, op32 = 0, oG32 = 0, oH32 = 0, oRi32 = 0, oCs = 0, otmp = 0,
          oYr = 0, oev = 0, orl32 = 0;
  RitzLayout rl32{};
  if (refine) {
    oUp = take(n * kb * 8); oZs64 = take(n * kb * 8); oW64 = take(n * kb * 8); oT64 = take(m * kb * 8);
    op32 = take((int64_t)nparts * kb * kb * 8); oG32 = take(kb * kb * 8); oH32 = take(kb * kb * 8);
    oRi32 = take(kb * kb * 8); oCs = take(kb * kb * 8); otmp = take(kb * kb * 8); oYr = take(kb * kb * 8);
    oev = take(kb * 8);
    rl32 = ritz_layout(nullptr, kb, kb);
    orl32 = take(rl32.bytes);
  }
  w.bytes = o;
  if (!base) return w;
  w.Q = base + oQ; w.Q2 = base + oQ2; w.Z = base + oZ; w.Zs = base + oZs; w.W = base + oW; w.T = base + oT;
  w.part = (double*)(base + opart); w.C1 = (double*)(base + oC1); w.C2 = (double*)(base + oC2);
  w.G = (double*)(base + oG); w.R1 = (double*)(base + oR1); w.R2 = (double*)(base + oR2);
  w.Rinv = (double*)(base + oRi); w.Rout = (double*)(base + oRo); w.H = (double*)(base + oH);
  w.ctl = (double*)(base + octl); w.theta_keep = (double*)(base + oth); w.Yk = (double*)(base + oYk);
  w.Bc = (double*)(base + oBc); w.Yf = (double*)(base + oYf); w.evals_f = (double*)(base + oef);
  w.res_f = (double*)(base + orf); w.counter = (unsigned*)(base + ocnt);
  w.ord = (int*)(base + oord); w.sel = (int*)(base + osel); w.row_of = (int*)(base + orow);
  w.ritz = ritz_layout(base + orl, M, M);
  if (refine) {
    w.Up = (double*)(base + oUp); w.Zs64 = (double*)(base + oZs64); w.W64 = (double*)(base + oW64);
    w.T64 = (double*)(base + oT64); w.part32 = (double*)(base + op32); w.G32 = (double*)(base + oG32);
    w.H32 = (double*)(base + oH32); w.Ri = (double*)(base + oRi32); w.Cs = (double*)(base + oCs);
    w.tmp = (double*)(base + otmp); w.Yr = (double*)(base + oYr); w.ev32 = (double*)(base + oev);
    w.ritz32 = ritz_layout(base + orl32, kb, kb);
  }
  return w;
}

int default_variant(int code, int which) {
  if (code == 0) return which == 0 ? kDyn + 7 : 6;  // measured best at 100k x 500k, block 8
  return 1;
}

// One operator application W = A Z (Zs = a ⊙ Z precomputed, T: m x B scratch)
// with the given SpMM kernels; launches and (optionally) events are counted.
struct Apply {
  const sg_gram_op* op;
  cudaStream_t s;
  int* status;
  unsigned* counter;
  bool timed;
  std::vector<cudaEvent_t> ev;
  int64_t launches = 0, spmm_launches = 0;

  int pass(int which, int variant, int code, int B, const void* in, void* out, const void* y) {
    const bool t = which == 0;
    const int64_t rows = t ? op->m : op->n;
    const int64_t* ptr = t ? op->colptr : op->indptr;
    const int32_t* idx = t ? op->rowidx : op->indices;
    const float* val = t ? op->cvalues : op->values;
    const void* scale = code ? (const void*)(t ? op->w2 : op->a) : (const void*)(t ? op->w2_f32 : op->a_f32);
    const void* dsh = t ? nullptr : (code ? (const void*)op->dinv : (const void*)op->dinv_f32);
    const void* yy = t ? nullptr : y;
    if (variant >= kDyn && code != 0) variant -= kDyn;  // the dynamic schedule is FP32 only
    int e;
    if (variant >= kDyn && t && op->order_t && op->order_t_positions > 0) {
      e = sg_spmm_dyn_ordered(code, B, op->order_t_positions, ptr, idx, val, in, out, scale, dsh, yy,
                              variant - kDyn, op->order_t, counter + which, s);
    } else if (variant >= kDyn) {
      e = sg_spmm_dyn(code, B, rows, ptr, idx, val, in, out, scale, dsh, yy, variant - kDyn, nullptr,
                      counter + which, s);
    } else if (variant >= kStaged) {
      const void* table = t ? op->staged_table_t : op->staged_table_x;
      if (!table) return SG_ERR_ARG;
      e = sg_spmm_staged(code, B, rows, t ? op->n : op->m, ptr, idx, val, table, in, out, scale, dsh, yy,
                         variant - kStaged, nullptr, status, s);
    } else {
      e = sg_spmm_masked(code, B, rows, ptr, idx, val, in, out, scale, dsh, yy, -1, variant, nullptr, s);
    }
    ++launches;
    ++spmm_launches;
    return e;
  }

  int apply(int code, int B, int vt, int vx, const void* Z, const void* Zs, void* T, void* W) {
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    if (timed) {
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventCreate(&e2);
      ev.push_back(e0);
      ev.push_back(e1);
      ev.push_back(e2);
      cudaEventRecord(e0, s);
    }
    int e = pass(0, vt, code, B, Zs, T, nullptr);
    if (e) return e;
    if (timed) cudaEventRecord(e1, s);
    e = pass(1, vx, code, B, T, W, Z);
    if (timed) cudaEventRecord(e2, s);
    return e;
  }

  void collect(double* ms_t, double* ms_x) {
    double a = 0.0, b = 0.0;
    for (size_t i = 0; i + 2 < ev.size(); i += 3) {
      float x = 0.f, y = 0.f;
      cudaEventElapsedTime(&x, ev[i], ev[i + 1]);
      cudaEventElapsedTime(&y, ev[i + 1], ev[i + 2]);
      a += x;
      b += y;
    }
    for (cudaEvent_t e : ev) cudaEventDestroy(e);
    ev.clear();
    *ms_t = a;
    *ms_x = b;
  }
};

int proj_launches(int code, int b, int ncols) {
  const int slice = (b * (code ? 8 : 4) >= 128 ? 1 : 2) * 256;
  return 2 * ((ncols + slice - 1) / slice);
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int64_t sg_lanczos_work_bytes(int precision, int block, int k, int64_t n, int64_t m, int basis, int keep) {
  (void)keep;
  if ((precision != 0 && precision != 1) || (block != 4 && block != 8 && block != 16 && block != 32) || k < 1 ||
      n < 2 || m < 1)
    return -1;
  Basis bs = default_basis(k, block);
  int M = basis > 0 ? basis : bs.M;
  M = (int)std::min<int64_t>(M, (n - block) / block * block);
  if (M < block || M + block > kRitzMaxN) return -1;
  return layout(nullptr, precision, block, k, n, m, M, sg_proj_parts()).bytes;
}

extern "C" int sg_lanczos(const sg_gram_op* op, int precision, int block, int k, uint64_t seed,
                          const sg_lanczos_opts* opts, void* work, int64_t work_bytes, double* evals, double* evecs,
                          double* residuals, sg_lanczos_info* info, int* status, void* stream) {
  if (!op || !work || !evals || !evecs || !status || (precision != 0 && precision != 1)) return SG_ERR_ARG;
  if (block != 4 && block != 8 && block != 16 && block != 32) return SG_ERR_ARG;
  const int64_t n = op->n, m = op->m;
  if (n < 2 || m < 1 || k < 1 || k >= n) return SG_ERR_ARG;
  if (((uintptr_t)work & 255u) != 0) return SG_ERR_ARG;
  const int code = precision;
  const int b = block;
  sg_lanczos_opts o{};
  if (opts) {
    o = *opts;
  } else {  // library defaults: every pair's vector to tol_vec, correction sweep on, default kernels
    o.refine = 1;
    o.max_restarts = -1;
    o.variant_t = o.variant_x = o.refine_variant_t = o.refine_variant_x = -1;
  }
  // 3e-9: at 100,000 cells x 500,000 features the wanted eigenvalues end in a
  // dense cluster of small ones (relative gaps ~2e-4) that the k-th / (k+1)-th
  // boundary cuts; with 1e-8 the returned vectors of that cluster stayed up to
  // 1.6e-4 rad from a solution converged to 1e-12 (block 16), with 3e-9
  // within 3e-5 rad (block 8: 5.3e-5)
  const double tol_vec = o.tol_vec > 0 ? o.tol_vec : 3e-9;
  const double tol_val = o.tol_val > 0 ? o.tol_val : 1e-6;
  const int max_restarts = o.max_restarts >= 0 ? o.max_restarts : 200;
  const int vt = o.variant_t >= 0 ? o.variant_t : default_variant(code, 0);
  const int vx = o.variant_x >= 0 ? o.variant_x : default_variant(code, 1);
  // correction sweep: refine 1 = compensated FP32 kernels (variants of sg_spmm_ds: dynamic rows and
  // two index chunks in flight, the fastest for both passes at 100k and 1M cells), 2 = FP64 kernels
  const bool ds_sweep = o.refine != 2;
  const int rvt = o.refine_variant_t >= 0 ? o.refine_variant_t : (ds_sweep ? 3 : default_variant(1, 0));
  const int rvx = o.refine_variant_x >= 0 ? o.refine_variant_x : (ds_sweep ? 3 : default_variant(1, 1));
  if (ds_sweep && (rvt > 3 || rvx > 3)) return SG_ERR_ARG;
  Basis bs = default_basis(k, b);
  int M = o.basis > 0 ? o.basis : bs.M;
  int keep = o.keep > 0 ? o.keep : bs.keep;
  M = (int)std::min<int64_t>(M, (n - b) / b * b);
  keep = std::min(keep, M - b);
  if (keep < k || M % b || M < b || M + b > kRitzMaxN) return SG_ERR_ARG;
  const int ld = M + b;
  const int nparts = sg_proj_parts();
  Work w = layout((char*)work, code, b, k, n, m, M, nparts);
  if (work_bytes < w.bytes) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  const void* a = code ? (const void*)op->a : (const void*)op->a_f32;
  Apply ap{op, s, status, w.counter, o.time_spmm != 0, {}};
  int64_t& nl = ap.launches;
  double ph_cycles = 0.0, ph_ritz = 0.0, ph_restart = 0.0, ph_refine = 0.0;
#define SG_TRY(x)              \
  do {                         \
    const int e__ = (x);       \
    if (e__) return e__;       \
  } while (0)
  if (cudaMemsetAsync(status, 0, sizeof(int), s) != cudaSuccess ||
      cudaMemsetAsync(w.H, 0, sizeof(double) * ld * ld, s) != cudaSuccess)
    return SG_ERR_CUDA;
  auto cholqr2 = [&]() -> int {
    SG_TRY(sg_block_cholqr(code, b, n, w.W, w.part, nparts, w.G, w.R1, w.Rinv, status, s));
    SG_TRY(sg_block_cholqr(code, b, n, w.W, w.part, nparts, w.G, w.R2, w.Rinv, status, s));
    nl += 8;
    return SG_OK;
  };
  // start block: deterministic uniform noise, orthonormalised
  SG_TRY(sg_fill_random(code, n * b, seed, w.W, s));
  ++nl;
  SG_TRY(cholqr2());
  SG_TRY(sg_block_finish(code, b, n, w.W, w.Q, ld, 0, w.Z, w.Zs, a, s));
  ++nl;
  int mcols = 0;
  int64_t n_mv = 0;
  int restarts = 0;
  std::vector<double> hist;
  double ctl[8] = {0};
  int Me = 0, nw = 0;
  bool converged = false;
  char* Q = w.Q;
  char* Q2 = w.Q2;
  while (true) {
    const double tc = now_s();
    while (mcols + b <= M) {
      SG_TRY(ap.apply(code, b, vt, vx, w.Z, w.Zs, w.T, w.W));
      ++n_mv;
      const int ncols = mcols + b;
      for (double* C : {w.C1, w.C2}) {
        SG_TRY(sg_block_proj(code, b, n, Q, ld, ncols, w.W, w.part, nparts, C, s));
        SG_TRY(sg_block_update(code, b, n, Q, ld, ncols, C, w.W, s));
        nl += proj_launches(code, b, ncols) + 1;
      }
      SG_TRY(cholqr2());
      SG_TRY(sg_lanczos_hblock(b, w.H, ld, mcols, w.C1, w.C2, w.R1, w.R2, w.Rout, 1, s));
      SG_TRY(sg_block_finish(code, b, n, w.W, Q, ld, mcols + b, w.Z, w.Zs, a, s));
      nl += 2;
      mcols += b;
    }
    Me = mcols;  // after a thick restart keep need not be a multiple of b
    const double tr = now_s();
    ph_cycles += tr - tc;
    // Rayleigh-Ritz on the GPU: the keep + 4 largest and smallest eigenvalues
    // of H[:Me, :Me] (the largest magnitudes are among them), eigenvectors of
    // the keep of largest magnitude
    const int want = std::min(Me, keep + 4);
    SG_TRY(ritz_values(Me, w.H, ld, want, want, w.ritz, &nw, s));
    order_kernel<<<1, 512, sizeof(int) * nw, s>>>(nw, w.ritz.lam, keep, w.ord, w.sel, w.row_of);
    SG_CHECK_LAUNCH();
    SG_TRY(ritz_vectors(Me, w.ritz, w.sel, keep, s));
    select_kernel<<<1, 512, 12 * (size_t)k, s>>>(Me, nw, w.ritz.lam, w.ord, w.row_of, w.ritz.Zt, w.H, ld, b, k, keep,
                                                 tol_vec, tol_val, o.vec_positive_only != 0, status, w.ctl,
                                                 w.theta_keep, w.Yk, w.Bc, w.Yf, w.evals_f, w.res_f);
    SG_CHECK_LAUNCH();
    nl += 9;
    if (cudaMemcpyAsync(ctl, w.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return SG_ERR_CUDA;
    const double tq = now_s();
    ph_ritz += tq - tr;
    if ((int)ctl[3] != 0) return (int)ctl[3];  // rank-deficient Krylov block (or a staged-SpMM timeout)
    const double worst = ctl[0], anorm = ctl[2];
    hist.push_back(ctl[1]);
    converged = worst <= 1.0;
    if (converged || restarts >= max_restarts) break;
    // FP32 floor: the residuals stopped falling while already within a few
    // hundred FP32 ulps of |A| (slow convergence above that keeps going)
    if (code == 0 && hist.size() >= 6) {
      const size_t h = hist.size();
      const double last3 = std::min(hist[h - 1], std::min(hist[h - 2], hist[h - 3]));
      double before = hist[0], all = hist[0];
      for (size_t i = 0; i < h; ++i) {
        if (i < h - 3) before = std::min(before, hist[i]);
        all = std::min(all, hist[i]);
      }
      if (last3 > 0.7 * before && all <= kFp32Floor * anorm) break;
    }
    ++restarts;
    SG_TRY(sg_basis_rotate(code, code, n, Q, ld, Me, w.Yk, keep, keep, Q2, ld, s));
    SG_TRY(sg_block_finish(code, b, n, w.Z, Q2, ld, keep, nullptr, nullptr, nullptr, s));
    hrestart_kernel<<<grid_for((int64_t)ld * ld, 256, 1024), 256, 0, s>>>(w.H, ld, ld, keep, b, w.theta_keep, w.Bc);
    SG_CHECK_LAUNCH();
    nl += 3;
    std::swap(Q, Q2);
    mcols = keep;
    ph_restart += now_s() - tq;
  }
  const double tf = now_s();
  double* ev_dev = w.evals_f;
  const int64_t solve_spmm = ap.spmm_launches;
  ap.timed = false;  // the event times cover the solve's own SpMM launches
  if (o.refine && code == 0 && k <= 32) {
    // Correction sweep over the k wanted Ritz vectors and the next ones in
    // |θ| order up to 32 (guard vectors): U = Q Yk[:, :kr], G = UᵀU and
    // Hm = Uᵀ A U in FP64-class arithmetic, generalized eigenproblem
    // Hm y = θ G y by Cholesky, the k of largest |θ| returned.  The guards
    // let the sweep separate a wanted pair from an unwanted one close to it
    // (the k-th and (k+1)-th eigenvalues of a tight cluster), which a sweep
    // over the k vectors alone cannot.
    const int kb = 32;
    const int kr = std::min(kb, keep);
    if (kr < kb && cudaMemsetAsync(w.Up, 0, sizeof(double) * n * kb, s) != cudaSuccess) return SG_ERR_CUDA;
    SG_TRY(sg_basis_rotate(code, 1, n, Q, ld, Me, w.Yk, keep, kr, w.Up, kb, s));
    SG_TRY(sg_block_proj(1, kb, n, w.Up, kb, kb, w.Up, w.part32, nparts, w.G32, s));
    if (ds_sweep) {
      // Zs64 / T64 hold (hi, lo) FP32 pairs here: the same bytes as FP64
      SG_TRY(sg_ds_split(n, op->a, w.Up, w.Zs64, s));
      const bool ordered = rvt >= 2 && op->order_t && op->order_t_positions > 0;
      SG_TRY(sg_spmm_ds(0, ordered ? op->order_t_positions : m, op->colptr, op->rowidx, op->cvalues, w.Zs64, w.T64,
                        op->w2, nullptr, nullptr, rvt, ordered ? op->order_t : nullptr, w.counter, s));
      SG_TRY(sg_spmm_ds(1, n, op->indptr, op->indices, op->values, w.T64, w.W64, op->a, op->dinv, w.Up, rvx,
                        nullptr, w.counter + 1, s));
      nl += 3;
    } else {
      SG_TRY(sg_block_finish(1, kb, n, w.Up, nullptr, 0, 0, nullptr, w.Zs64, op->a, s));
      SG_TRY(ap.apply(1, kb, rvt, rvx, w.Up, w.Zs64, w.T64, w.W64));
      ++nl;
    }
    SG_TRY(sg_block_proj(1, kb, n, w.Up, kb, kb, w.W64, w.part32, nparts, w.H32, s));
    refine_prep_kernel<<<1, 256, 0, s>>>(kr, kb, w.G32, w.H32, w.Ri, w.Cs, w.tmp, status);
    SG_CHECK_LAUNCH();
    nl += 2 + 2 * proj_launches(1, kb, kb);
    int nw2 = 0;
    SG_TRY(ritz_values(kr, w.Cs, kr, kr, kr, w.ritz32, &nw2, s));
    SG_TRY(ritz_vectors(kr, w.ritz32, nullptr, nw2, s));
    nl += 7;
    refine_finish_kernel<<<1, 256, 0, s>>>(k, kr, w.Ri, w.ritz32.lam, w.ritz32.Zt, w.Yr, w.ev32);
    SG_CHECK_LAUNCH();
    SG_TRY(sg_basis_rotate(1, 1, n, w.Up, kb, kr, w.Yr, k, k, evecs, k, s));
    nl += 2;
    ev_dev = w.ev32;
  } else {
    // Ritz vectors (FP64 output), eigenvalues descending like the reference
    SG_TRY(sg_basis_rotate(code, 1, n, Q, ld, Me, w.Yf, k, k, evecs, k, s));
    ++nl;
  }
  std::vector<double> res_h(k);
  int st = 0;
  if (cudaMemcpyAsync(evals, ev_dev, sizeof(double) * k, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(res_h.data(), w.res_f, sizeof(double) * k, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaMemcpyAsync(&st, status, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return SG_ERR_CUDA;
  if (st) return st;
  ph_refine = now_s() - tf;
  if (residuals)
    for (int i = 0; i < k; ++i) residuals[i] = res_h[i];
  double ms_t = 0.0, ms_x = 0.0;
  ap.collect(&ms_t, &ms_x);
  if (info) {
    sg_lanczos_info I{};
    I.block_matvecs = n_mv;
    I.restarts = restarts;
    I.converged = converged ? 1 : 0;
    I.basis = M;
    I.keep = keep;
    double mr = 0.0;
    for (int i = 0; i < k; ++i) mr = std::max(mr, res_h[i]);
    I.max_residual = mr;
    for (int q = 0; q < 4; ++q) I.next_evals[q] = ctl[4 + q];
    I.seconds_cycles = ph_cycles;
    I.seconds_ritz = ph_ritz;
    I.seconds_restart = ph_restart;
    I.seconds_refine = ph_refine;
    I.spmm_ms_t = ms_t;
    I.spmm_ms_x = ms_x;
    I.spmm_launches = solve_spmm;
    I.kernel_launches = nl;
    *info = I;
  }
#undef SG_TRY
  return SG_OK;
}
