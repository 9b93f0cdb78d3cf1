// Dense symmetric FP64 eigensolver on the GPU: the Rayleigh-Ritz step of the
// block Krylov-Schur solver (sg_lanczos), which replaces the small eigenproblem
// ARPACK solves inside the reference's eigsh call
// (snapatac2-python/src/embedding.rs:155-171).
//
// GB300 runs FP64 at about two fused multiply-adds per clock per SM, so one
// CTA would need milliseconds for the O(n^3) reduction of a 200 x 200 matrix
// and tens of milliseconds at 576 x 576.  The work is spread instead:
//
//   tridiag    Householder reduction A = Q T Qᵀ on one thread-block cluster
//              (up to 16 CTAs).  Row i of A lives in the shared memory of CTA
//              i mod CS; each step broadcasts the reflector and the product
//              p = τ A v through distributed shared memory, with two cluster
//              barriers per step (buffers alternate between steps).
//   bisect     eigenvalues of T by multisection on Sturm counts: one warp per
//              wanted eigenvalue, 32 shifts per round, to absolute accuracy
//              eps·‖T‖ (LAPACK dstebz's default).
//   invit      eigenvectors of T by inverse iteration with a pivoted
//              tridiagonal LU (as LAPACK dstein): one warp per cluster of
//              near-degenerate eigenvalues (1e-9 ‖T‖), modified Gram-Schmidt
//              inside a cluster.
//   orth       one FP64 Cholesky-QR of all the vectors (Gram matrix by
//              warps across the GPU, factor and triangular solve in one CTA):
//              separately iterated vectors of eigenvalues 1e-9..1e-3 ‖T‖
//              apart are orthogonal only to eps ‖T‖ / gap; rotating them by
//              that much moves their residuals by ~eps ‖T‖.
//   backtr     eigenvectors of A = Q z: one warp per vector applies the
//              reflectors in reverse order.
//
// Every sum runs in a fixed order, so results are reproducible run to run.
#include <cooperative_groups.h>
#include <float.h>

#include <atomic>

#include "common.cuh"
#include "internal.h"

namespace cg = cooperative_groups;

namespace sg {
namespace {

constexpr int kTriThreads = 256;
constexpr int kMaxCluster = 16;

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Shared memory of the reduction: rows [R][n], v[2][n], p[2][n], 2 x 32
// slots (per-CTA partial sums of pᵀv in 0..CS-1, τ in 16), 32 per-warp
// partials, 4 scalars.  v and the slots are double-buffered: the owner of
// step j + 1 writes them into the other CTAs before those have finished step
// j.  p is written by the other CTAs only after the step's first cluster
// barrier, so the p buffer of the other parity holds w = p + K v.
inline size_t tridiag_smem(int n, int CS) {
  const int R = (n + CS - 1) / CS;
  return ((size_t)R * n + 4 * (size_t)n + 64 + 32 + 4) * sizeof(double);
}

// GB300 runs FP64 at about two lanes per clock per SM, so a warp-wide FP64
// instruction holds its SM sub-partition for tens of clocks: the scalar steps
// (the reflector's norm, square root and divisions, the K factor) run once,
// on one thread or one warp, and are passed on through shared memory; the
// vector w = p + K v is formed once per step, and each trailing element is
// updated by two FMAs.
template <int CS>
__global__ void __launch_bounds__(kTriThreads)
tridiag_kernel(int n, const double* __restrict__ A, int64_t lda, double* __restrict__ d, double* __restrict__ e,
               double* __restrict__ tau, double* __restrict__ V) {
  cg::cluster_group cl = cg::this_cluster();
  const int rank = CS > 1 ? (int)cl.block_rank() : 0;
  extern __shared__ double smem_d[];
  const int R = (n + CS - 1) / CS;
  double* Al = smem_d;
  double* vb = Al + (size_t)R * n;
  double* pb = vb + 2 * n;
  double* slots = pb + 2 * n;
  double* red = slots + 64;
  double* sc = red + 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int t = threadIdx.x; t < R * n; t += blockDim.x) {
    const int li = t / n, c = t % n;
    const int i = li * CS + rank;
    Al[t] = i < n ? A[(int64_t)i * lda + c] : 0.0;
  }
  if (CS > 1) cl.sync(); else __syncthreads();
  for (int j = 0; j + 2 < n; ++j) {
    const int par = j & 1;
    double* v = vb + par * n;
    double* p = pb + par * n;
    double* wv = pb + (par ^ 1) * n;
    double* sl = slots + par * 32;
    if (rank == j % CS) {
      // reflector of column j (= row j) below the diagonal, LAPACK dlarfg style
      const double* row = Al + (size_t)(j / CS) * n;
      double s = 0.0;
      for (int k = j + 2 + threadIdx.x; k < n; k += blockDim.x) s = fma(row[k], row[k], s);
      s = warp_sum_d(s);
      if (lane == 0) red[warp] = s;
      __syncthreads();
      if (threadIdx.x == 0) {
        double sigma = 0.0;
        for (int w = 0; w < nwarps; ++w) sigma += red[w];
        const double alpha = row[j + 1];
        double tj = 0.0, beta = alpha, scale = 0.0;
        if (sigma > 0.0) {
          const double mu = sqrt(fma(alpha, alpha, sigma));
          beta = alpha <= 0.0 ? mu : -mu;
          // τ = (β - α)/β and 1/(α - β) from one reciprocal
          const double am = alpha - beta;
          const double inv = 1.0 / (beta * am);
          tj = -am * am * inv;
          scale = beta * inv;
        }
        sc[0] = tj;
        sc[1] = scale;
        sl[16] = tj;
        d[j] = row[j];
        e[j] = beta;
        tau[j] = tj;
      }
      __syncthreads();
      const double scale = sc[1];
      for (int k = j + 1 + threadIdx.x; k < n; k += blockDim.x) {
        const double vk = k == j + 1 ? 1.0 : row[k] * scale;
        v[k] = vk;
        V[(int64_t)j * n + k] = vk;
      }
      __syncthreads();
      if (CS > 1) {
        for (int r = 0; r < CS; ++r) {
          if (r == rank) continue;
          double* rv = cl.map_shared_rank(v, r);
          for (int k = j + 1 + threadIdx.x; k < n; k += blockDim.x) rv[k] = v[k];
          if (threadIdx.x == 0) cl.map_shared_rank(sl, r)[16] = sc[0];
        }
      }
    }
    if (CS > 1) cl.sync(); else __syncthreads();
    // p_i = τ Σ_k A[i][k] v_k over the trailing rows this CTA owns (warp per row)
    const double tj = sl[16];
    const int first = j + 1 - rank;
    const int li0 = first <= 0 ? 0 : (first + CS - 1) / CS;
    double sv = 0.0;
    for (int li = li0 + warp; li < R; li += nwarps) {
      const int i = li * CS + rank;
      if (i >= n) break;
      const double* row = Al + (size_t)li * n;
      double acc = 0.0;
      for (int k = j + 1 + lane; k < n; k += 32) acc = fma(row[k], v[k], acc);
      acc = warp_sum_d(acc) * tj;
      sv = fma(acc, v[i], sv);
      if (lane < CS) (CS > 1 ? cl.map_shared_rank(p, lane) : p)[i] = acc;
    }
    if (lane == 0) red[warp] = sv;
    __syncthreads();
    if (threadIdx.x < CS) {
      double s2 = 0.0;
      for (int w = 0; w < nwarps; ++w) s2 += red[w];
      (CS > 1 ? cl.map_shared_rank(sl, (int)threadIdx.x) : sl)[rank] = s2;
    }
    if (CS > 1) cl.sync(); else __syncthreads();
    // K = -τ/2 pᵀv (one warp), w = p + K v (once), A <- A - v wᵀ - w vᵀ on
    // the owned trailing rows
    if (warp == 0) {
      const double x = warp_sum_d(lane < CS ? sl[lane] : 0.0);
      if (lane == 0) sc[3] = -0.5 * tj * x;
    }
    __syncthreads();
    const double K = sc[3];
    for (int k = j + 1 + threadIdx.x; k < n; k += blockDim.x) wv[k] = fma(K, v[k], p[k]);
    __syncthreads();
    for (int li = li0 + warp; li < R; li += nwarps) {
      const int i = li * CS + rank;
      if (i >= n) break;
      double* row = Al + (size_t)li * n;
      const double vi = v[i], wi = wv[i];
      for (int k = j + 1 + lane; k < n; k += 32) row[k] = fma(-vi, wv[k], fma(-wi, v[k], row[k]));
    }
    __syncthreads();
  }
  // the last 2 x 2 block
  if (threadIdx.x == 0) {
    if (n >= 2 && rank == (n - 2) % CS) {
      const double* row = Al + (size_t)((n - 2) / CS) * n;
      d[n - 2] = row[n - 2];
      e[n - 2] = row[n - 1];
      tau[n - 2] = 0.0;
    }
    if (rank == (n - 1) % CS) {
      d[n - 1] = Al[(size_t)((n - 1) / CS) * n + n - 1];
      tau[n - 1] = 0.0;
    }
  }
  if (CS > 1) cl.sync();
}

// Gershgorin interval, ‖T‖ (max absolute row sum) and the pivot floor of the
// Sturm recurrence (LAPACK: safe minimum x max(1, max e²)); one warp.
struct TriBounds {
  double lo, hi, tnorm, pivmin;
};

__device__ TriBounds tri_bounds_warp(int n, const double* __restrict__ d, const double* __restrict__ e) {
  const int lane = threadIdx.x & 31;
  double lo = DBL_MAX, hi = -DBL_MAX, tn = 0.0, e2 = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    tn = fmax(tn, fabs(d[i]) + r);
    if (i + 1 < n) e2 = fmax(e2, e[i] * e[i]);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
    e2 = fmax(e2, __shfl_xor_sync(0xffffffffu, e2, o));
  }
  TriBounds b;
  b.tnorm = tn;
  b.pivmin = DBL_MIN * fmax(1.0, e2);
  const double pad = 2.0 * DBL_EPSILON * tn + 2.0 * b.pivmin;
  b.lo = lo - pad;
  b.hi = hi + pad;
  return b;
}

// Number of eigenvalues of T below x (e2 = squared off-diagonal), as the
// number of sign changes of the Sturm sequence of leading principal minors
// p_i = (d_i - x) p_{i-1} - e²_{i-1} p_{i-2} (Givens; Wilkinson, The
// Algebraic Eigenvalue Problem, 5.37-5.45): q_i = p_i / p_{i-1} <= 0 exactly
// when p_i and p_{i-1} differ in sign.  This form has no division: GB300
// runs an FP64 division as a chain of dependent FP64 operations (several
// hundred clocks), so the ratio form q_i = (d_i - x) - e²/q_{i-1} costs about
// four times as much per step.  The pair (p_i, p_{i-1}) is rescaled by an
// exact power of two whenever its larger exponent leaves [2^-400, 2^400], so
// it neither overflows nor underflows.  A zero minor is replaced by a tiny
// value of the sign opposite to its predecessor, which counts it as
// negative, as the ratio form's pivot floor does.  Signs and exponents are
// read as integers, off the FP64 pipe.
__device__ __forceinline__ int sturm_count(int n, const double* __restrict__ d, const double* __restrict__ e2,
                                           double x) {
  constexpr long long kSign = (long long)0x8000000000000000ull;
  double pm = 1.0;
  double p = d[0] - x;
  if (p == 0.0) p = -DBL_MIN;
  int c = p < 0.0;
  for (int i = 1; i < n; ++i) {
    double pn = fma(-e2[i - 1], pm, (d[i] - x) * p);
    long long bn = __double_as_longlong(pn);
    const long long bp = __double_as_longlong(p);
    if ((bn & ~kSign) == 0) {  // zero minor: opposite sign to p, 2^-600 of the pair's scale (a normal number)
      const double mag = fmax(fabs(p), fabs(pm)) * 0x1p-600;
      pn = bp < 0 ? mag : -mag;
      bn = __double_as_longlong(pn);
    }
    c += (int)(((unsigned long long)(bn ^ bp)) >> 63);
    pm = p;
    p = pn;
    const int ex = (int)((bn >> 52) & 0x7ff), ey = (int)((bp >> 52) & 0x7ff);
    const int emax = ex > ey ? ex : ey;
    if (emax > 1023 + 400 || emax < 1023 - 400) {
      // multiply both by 2^(1023 - emax), built from its bits
      const double sc = __longlong_as_double((long long)(2046 - emax) << 52);
      p *= sc;
      pm *= sc;
    }
  }
  return c;
}

// lam[w] = eigenvalue of ascending rank ranks[w].  A group of kBisLanes lanes
// per wanted value evaluates kBisLanes shifts per round (multisection into
// kBisLanes + 1 parts).  A warp's FP64 instructions run one after another on
// its sub-partition's FP64 unit whatever the number of active lanes, so the
// time is rounds x steps x FP64 operations per step of one warp, with one
// warp per sub-partition (two-warp blocks).  d and e² are staged in shared
// memory.
constexpr int kBisLanes = 32;
constexpr int kBisThreads = 64;
__global__ void __launch_bounds__(kBisThreads)
bisect_kernel(int n, const double* __restrict__ d, const double* __restrict__ e, const int* __restrict__ ranks, int nw,
              double* __restrict__ lam) {
  __shared__ double ds[kRitzMaxN], e2s[kRitzMaxN];
  __shared__ TriBounds bs;
  if (threadIdx.x < 32) {
    const TriBounds b = tri_bounds_warp(n, d, e);
    if (threadIdx.x == 0) bs = b;
  }
  __syncthreads();
  // T and the shifts scaled by the power of two that brings ‖T‖ into [0.5, 1):
  // exact, and it bounds the growth of the minors per step
  const long long tb = __double_as_longlong(bs.tnorm);
  const int te = (int)((tb >> 52) & 0x7ff);
  const double sc = bs.tnorm > 0.0 && te > 0 ? __longlong_as_double((long long)(2045 - te) << 52) : 1.0;
  const double isc = bs.tnorm > 0.0 && te > 0 ? __longlong_as_double((long long)(te + 1) << 52) : 1.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    ds[i] = d[i] * sc;
    const double es = i + 1 < n ? e[i] * sc : 0.0;
    e2s[i] = es * es;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  constexpr int GPW = 32 / kBisLanes;
  const int g = lane / kBisLanes, gl = lane % kBisLanes;
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * GPW + g;
  if ((int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5) * GPW >= nw) return;  // whole warp idle
  const bool active = w < nw;
  const int r = active ? ranks[w] : 0;
  constexpr double kStep = 1.0 / (kBisLanes + 1);
  const double tnorm = bs.tnorm * sc;
  double lo = bs.lo * sc, hi = bs.hi * sc;
  const unsigned gmask = kBisLanes == 32 ? 0xffffffffu : ((1u << (kBisLanes % 32)) - 1u) << (g * kBisLanes);
  for (int it = 0; it < 64; ++it) {
    const double width = hi - lo;
    const bool done = !active || width <= 0.0 ||
                      width <= fmax(DBL_EPSILON * tnorm, 2.0 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)));
    if (__all_sync(0xffffffffu, done)) break;
    int c = 0;
    if (!done) c = sturm_count(n, ds, e2s, lo + width * ((gl + 1) * kStep));
    const unsigned above = (__ballot_sync(0xffffffffu, c > r) & gmask) >> ((g * kBisLanes) % 32);
    if (!done) {
      const int l = above ? __ffs(above) - 1 : kBisLanes;
      const double nlo = l == 0 ? lo : lo + width * (l * kStep);
      const double nhi = l == kBisLanes ? hi : lo + width * ((l + 1) * kStep);
      lo = nlo;
      hi = nhi;
    }
  }
  if (active && gl == 0) lam[w] = 0.5 * (lo + hi) * isc;
}

__device__ __forceinline__ double hash_unit(uint64_t a, uint64_t b) {
  uint64_t x = a * 0x9e3779b97f4a7c15ull + b + 0x632be59bd9b4e019ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  x ^= x >> 31;
  return (double)(x >> 11) * (2.0 / 9007199254740992.0) - 1.0;  // [-1, 1)
}

// Eigenvectors of T for the selected eigenvalues: sel[0..nsel) are indices
// into (ranks, lam), ascending (identity when sel is null).  One warp per
// cluster of selected eigenvalues with consecutive ranks closer than
// 1e-9 ‖T‖ (near-degenerate pairs).  Outside a cluster a converged vector is
// within eps ‖T‖ / gap <= 2.2e-7 of its eigenvector, and orth_kernel then
// restores orthonormality; LAPACK dstein clusters at 1e-3 ‖T‖ instead,
// which chains the dense bulk of a Ritz spectrum (tiny eigenvalues 1e-7
// apart) into long sequential runs.  Inside a cluster the vectors are done in
// order, each orthogonalised against the cluster's earlier ones after every
// solve (the dot products and updates spread over the lanes).  The pivoted
// LU and the triangular solves run on lane 0.  lu: per-cluster scratch of 4n
// doubles + n pivot flags.  Zt row t = eigenvector of selection t (unit
// 2-norm, largest component positive).
__global__ void invit_kernel(int n, const double* __restrict__ d, const double* __restrict__ e,
                             const int* __restrict__ ranks, const double* __restrict__ lam,
                             const int* __restrict__ sel, int nsel, double* __restrict__ Zt,
                             double* __restrict__ lu, unsigned char* __restrict__ piv) {
  const int lane = threadIdx.x & 31;
  const int t = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (t >= nsel) return;
  double tnorm = 0.0;
  for (int i = lane; i < n; i += 32)
    tnorm = fmax(tnorm, fabs(d[i]) + (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < n ? fabs(e[i]) : 0.0));
#pragma unroll
  for (int o = 16; o; o >>= 1) tnorm = fmax(tnorm, __shfl_xor_sync(0xffffffffu, tnorm, o));
  const double ortol = 1e-9 * tnorm;
  auto idx = [&](int w) { return sel ? sel[w] : w; };
  auto joined = [&](int w) {  // selection w continues the cluster of w - 1
    return w > 0 && ranks[idx(w)] == ranks[idx(w - 1)] + 1 && lam[idx(w)] - lam[idx(w - 1)] <= ortol;
  };
  if (joined(t)) return;  // not the first vector of its cluster (warp-uniform)
  int end = t + 1;
  while (end < nsel && joined(end)) ++end;
  double* L = lu + (size_t)t * 4 * n;  // multipliers
  double* U0 = L + n;                  // reciprocal pivots
  double* U1 = U0 + n;
  double* U2 = U1 + n;
  unsigned char* P = piv + (size_t)t * n;
  const double eps = DBL_EPSILON;
  const double tiny = eps * fmax(tnorm, DBL_MIN);
  double prev = 0.0;
  for (int w = t; w < end; ++w) {
    double x = lam[idx(w)];
    const double pertol = 10.0 * fabs(eps * x) + tiny;
    if (w > t && x - prev < pertol) x = prev + pertol;  // separate equal shifts, as dstein
    prev = x;
    double* z = Zt + (size_t)w * n;
    if (lane == 0) {
      // pivoted LU of T - x I: U has two superdiagonals; U0 keeps the
      // reciprocal of each pivot (tiny pivots replaced by ±eps‖T‖, as
      // dlagts does), so the solves below divide nothing
      double cd = d[0] - x, cs = n > 1 ? e[0] : 0.0;
      for (int i = 0; i + 1 < n; ++i) {
        const double sub = e[i], dn = d[i + 1] - x, sp = i + 2 < n ? e[i + 1] : 0.0;
        double pv;
        // one reciprocal per row (an FP64 division is a long chain of FP64
        // operations here): the multiplier is formed from the pivot's
        // reciprocal
        if (fabs(cd) >= fabs(sub)) {
          pv = cd;
          if (fabs(pv) < tiny) pv = pv < 0.0 ? -tiny : tiny;
          const double rp = 1.0 / pv;
          const double l = cd != 0.0 ? sub * rp : 0.0;
          U0[i] = rp; U1[i] = cs; U2[i] = 0.0; L[i] = l; P[i] = 0;
          cd = dn - l * cs;
          cs = sp;
        } else {
          pv = sub;
          const double rp = 1.0 / pv;
          const double l = cd * rp;
          U0[i] = fabs(pv) < tiny ? (pv < 0.0 ? -1.0 / tiny : 1.0 / tiny) : rp;
          U1[i] = dn; U2[i] = sp; L[i] = l; P[i] = 1;
          cd = cs - l * dn;
          cs = -l * sp;
        }
      }
      if (fabs(cd) < tiny) cd = cd < 0.0 ? -tiny : tiny;
      U0[n - 1] = 1.0 / cd;
    }
    for (int i = lane; i < n; i += 32) z[i] = hash_unit((uint64_t)ranks[idx(w)], (uint64_t)i);
    __syncwarp();
    // iterate until the solve grows a unit vector by 1e-3 / (eps ‖T‖) (the
    // shift is then an eigenvalue to working accuracy), then once more, at
    // most five times (LAPACK dstein's scheme)
    double mx = 1.0;
    for (int it = 0, extra = 0; it < 5 && extra < 2; ++it) {
      // scale to unit max norm, then solve (T - x I) y = z in place (lane 0)
      const double sc = mx > 0.0 ? 1.0 / mx : 1.0;
      for (int i = lane; i < n; i += 32) z[i] *= sc;
      __syncwarp();
      if (lane == 0) {
        for (int i = 0; i + 1 < n; ++i) {
          if (P[i]) { const double tmp = z[i]; z[i] = z[i + 1]; z[i + 1] = tmp; }
          z[i + 1] -= L[i] * z[i];
        }
        for (int i = n - 1; i >= 0; --i) {
          double r = z[i];
          if (i + 1 < n) r -= U1[i] * z[i + 1];
          if (i + 2 < n) r -= U2[i] * z[i + 2];
          z[i] = r * U0[i];
        }
      }
      __syncwarp();
      for (int s2 = t; s2 < w; ++s2) {  // modified Gram-Schmidt inside the cluster
        const double* q = Zt + (size_t)s2 * n;
        double dot = 0.0;
        for (int i = lane; i < n; i += 32) dot = fma(q[i], z[i], dot);
        dot = warp_sum_d(dot);
        for (int i = lane; i < n; i += 32) z[i] = fma(-dot, q[i], z[i]);
        __syncwarp();
      }
      mx = 0.0;
      for (int i = lane; i < n; i += 32) mx = fmax(mx, fabs(z[i]));
#pragma unroll
      for (int o = 16; o; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
      if (extra > 0 || mx * tiny >= 1e-3) ++extra;
    }
    double nrm = 0.0, big = 0.0;
    int ib = n;
    for (int i = lane; i < n; i += 32) {
      nrm = fma(z[i], z[i], nrm);
      if (fabs(z[i]) > big) { big = fabs(z[i]); ib = i; }
    }
    nrm = warp_sum_d(nrm);
#pragma unroll
    for (int o = 16; o; o >>= 1) {  // the largest |component|, lowest index on ties
      const double bo = __shfl_xor_sync(0xffffffffu, big, o);
      const int io = __shfl_xor_sync(0xffffffffu, ib, o);
      if (bo > big || (bo == big && io < ib)) { big = bo; ib = io; }
    }
    double sc = nrm > 0.0 ? 1.0 / sqrt(nrm) : 0.0;
    if (ib < n && z[ib] < 0.0) sc = -sc;
    __syncwarp();
    for (int i = lane; i < n; i += 32) z[i] *= sc;
    __syncwarp();
  }
}

// G (lower triangle) = Zt Ztᵀ over the nw rows of length n; one warp per entry
__global__ void gram_rows_kernel(int nw, int n, const double* __restrict__ Zt, double* __restrict__ G) {
  const int lane = threadIdx.x & 31;
  const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int64_t tot = (int64_t)nw * (nw + 1) / 2;
  if (w >= tot) return;
  // w -> (i, j), j <= i
  int i = (int)((sqrt(8.0 * (double)w + 1.0) - 1.0) * 0.5);
  while ((int64_t)i * (i + 1) / 2 > w) --i;
  while ((int64_t)(i + 1) * (i + 2) / 2 <= w) ++i;
  const int j = (int)(w - (int64_t)i * (i + 1) / 2);
  const double* a = Zt + (size_t)i * n;
  const double* b = Zt + (size_t)j * n;
  double s = 0.0;
  for (int c = lane; c < n; c += 32) s = fma(a[c], b[c], s);
  s = warp_sum_d(s);
  if (lane == 0) G[(size_t)i * nw + j] = s;
}

// Cholesky G = L Lᵀ in place (lower), then Zt <- L⁻¹ Zt (rows orthonormal).
// One CTA; a non-positive pivot leaves Zt as it is.
__global__ void __launch_bounds__(1024) orth_kernel(int nw, int n, double* __restrict__ G, double* __restrict__ Zt) {
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < nw; ++j) {
    if (threadIdx.x == 0) {
      const double piv = G[(size_t)j * nw + j];
      if (!(piv > 0.0)) bad = 1;
      else G[(size_t)j * nw + j] = sqrt(piv);
    }
    __syncthreads();
    if (bad) return;
    const double ljj = G[(size_t)j * nw + j];
    for (int i = j + 1 + threadIdx.x; i < nw; i += blockDim.x) G[(size_t)i * nw + j] /= ljj;
    __syncthreads();
    // trailing update of the lower triangle: G[i][k] -= L[i][j] L[k][j],
    // j < k <= i; warp per row, lanes over k
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int i = j + 1 + warp; i < nw; i += nwarps) {
      const double lij = G[(size_t)i * nw + j];
      for (int k = j + 1 + lane; k <= i; k += 32) G[(size_t)i * nw + k] -= lij * G[(size_t)k * nw + j];
    }
    __syncthreads();
  }
  for (int c = threadIdx.x; c < n; c += blockDim.x) {  // forward substitution, one column per thread
    for (int i = 0; i < nw; ++i) {
      double y = Zt[(size_t)i * n + c];
      for (int q = 0; q < i; ++q) y -= G[(size_t)i * nw + q] * Zt[(size_t)q * n + c];
      Zt[(size_t)i * n + c] = y / G[(size_t)i * nw + i];
    }
  }
}

// Zt rows <- Q Zt rows, Q = H_0 H_1 ... H_{n-3}; one warp per vector
__global__ void backtr_kernel(int n, const double* __restrict__ V, const double* __restrict__ tau, int nw,
                              double* __restrict__ Zt) {
  extern __shared__ double zsh[];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  if (w >= nw) return;
  double* z = zsh + (size_t)wl * n;
  double* g = Zt + (size_t)w * n;
  for (int i = lane; i < n; i += 32) z[i] = g[i];
  __syncwarp();
  for (int j = n - 3; j >= 0; --j) {
    const double tj = tau[j];
    if (tj == 0.0) continue;
    const double* vj = V + (size_t)j * n;
    double s = 0.0;
    for (int k = j + 1 + lane; k < n; k += 32) s = fma(vj[k], z[k], s);
    s = warp_sum_d(s) * tj;
    for (int k = j + 1 + lane; k < n; k += 32) z[k] = fma(-s, vj[k], z[k]);
    __syncwarp();
  }
  for (int i = lane; i < n; i += 32) g[i] = z[i];
}

__global__ void ranks_kernel(int n, int p, int q, int* __restrict__ ranks) {
  // the q smallest and p largest ranks, ascending (all n when they overlap)
  const int nw = p + q >= n ? n : p + q;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nw; t += gridDim.x * blockDim.x)
    ranks[t] = (p + q >= n || t < q) ? t : n - p + (t - q);
}

// cluster size the reduction kernel launches with (0: not yet chosen; every
// thread that chooses finds the same value)
std::atomic<int> g_cluster_cs{0};

template <int CS>
int launch_tridiag_cs(int n, const double* A, int64_t lda, double* d, double* e, double* tau, double* V,
                      cudaStream_t s, bool probe_only) {
  const size_t smem = tridiag_smem(n, CS);
  if (smem > 227 * 1024) return SG_ERR_ARG;
  // the cap is set to the largest size any call needs, never to this call's:
  // calls on other host threads set the same value, so none can lower the
  // cap between another thread's set and its launch
  if (cudaFuncSetAttribute(tridiag_kernel<CS>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024) !=
      cudaSuccess)
    return SG_ERR_CUDA;
  if (CS > 8 && cudaFuncSetAttribute(tridiag_kernel<CS>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                    cudaSuccess)
    return SG_ERR_CUDA;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(CS, 1, 1);
  cfg.blockDim = dim3(kTriThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CS;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (probe_only) {
    int nc = 0;
    if (cudaOccupancyMaxActiveClusters(&nc, tridiag_kernel<CS>, &cfg) != cudaSuccess) {
      cudaGetLastError();
      return SG_ERR_CUDA;
    }
    return nc > 0 ? SG_OK : SG_ERR_CAP;
  }
  if (cudaLaunchKernelEx(&cfg, tridiag_kernel<CS>, n, A, lda, d, e, tau, V) != cudaSuccess) return SG_ERR_CUDA;
  return SG_OK;
}

int launch_tridiag_any(int cs, int n, const double* A, int64_t lda, double* d, double* e, double* tau, double* V,
                       cudaStream_t s, bool probe) {
  switch (cs) {
    case 16: return launch_tridiag_cs<16>(n, A, lda, d, e, tau, V, s, probe);
    case 8: return launch_tridiag_cs<8>(n, A, lda, d, e, tau, V, s, probe);
    case 4: return launch_tridiag_cs<4>(n, A, lda, d, e, tau, V, s, probe);
    case 2: return launch_tridiag_cs<2>(n, A, lda, d, e, tau, V, s, probe);
    case 1: return launch_tridiag_cs<1>(n, A, lda, d, e, tau, V, s, probe);
    default: return SG_ERR_ARG;
  }
}

}  // namespace

// The largest cluster size (16, 8, 4, 2, 1) whose CTAs hold the n-row
// matrix in shared memory and that this device can launch.
int ritz_cluster_size(int n) {
  for (int cs = kMaxCluster; cs >= 1; cs >>= 1) {
    if (tridiag_smem(n, cs) > 227 * 1024) break;  // smaller clusters hold more rows each
    if (launch_tridiag_any(cs, n, nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, true) == SG_OK)
      return cs;
  }
  return 0;
}

RitzLayout ritz_layout(char* base, int n, int nw) {
  RitzLayout L{};
  int64_t o = 0;
  auto take = [&](int64_t b) { const int64_t r = o; o += (b + 255) / 256 * 256; return r; };
  const int64_t od = take(8 * (int64_t)n), oe = take(8 * (int64_t)n), ot = take(8 * (int64_t)n),
                oV = take(8 * (int64_t)n * n), orr = take(4 * (int64_t)n), ol = take(8 * (int64_t)n),
                oz = take(8 * (int64_t)n * nw), olu = take(32 * (int64_t)n * nw), op = take((int64_t)n * nw),
                oG = take(8 * (int64_t)nw * nw);
  if (base) {
    L.d = (double*)(base + od);
    L.e = (double*)(base + oe);
    L.tau = (double*)(base + ot);
    L.V = (double*)(base + oV);
    L.ranks = (int*)(base + orr);
    L.lam = (double*)(base + ol);
    L.Zt = (double*)(base + oz);
    L.lu = (double*)(base + olu);
    L.piv = (unsigned char*)(base + op);
    L.G = (double*)(base + oG);
  }
  L.bytes = o;
  return L;
}

// Eigenvalues of the symmetric n x n matrix A (row-major, lda): the q
// smallest and p largest (all n when p + q >= n), ascending into L.lam, their
// ranks into L.ranks, the count into *nw.  Leaves the reduction (L.d, L.e,
// L.tau, L.V) for ritz_vectors.
int ritz_values(int n, const double* A, int64_t lda, int p, int q, const RitzLayout& L, int* nw, cudaStream_t s) {
  if (n < 1 || p < 0 || q < 0 || p + q < 1) return SG_ERR_ARG;
  const int cnt = p + q >= n ? n : p + q;
  *nw = cnt;
  int cs = g_cluster_cs.load();
  if (cs == 0 || tridiag_smem(n, cs) > 227 * 1024) {
    cs = ritz_cluster_size(n);
    if (cs == 0) return SG_ERR_CAP;
    g_cluster_cs.store(cs);
  }
  int err = launch_tridiag_any(cs, n, A, lda, L.d, L.e, L.tau, L.V, s, false);
  if (err) return err;
  ranks_kernel<<<grid_for(cnt, 256), 256, 0, s>>>(n, p, q, L.ranks);
  SG_CHECK_LAUNCH();
  bisect_kernel<<<grid_for((int64_t)cnt * kBisLanes, kBisThreads), kBisThreads, 0, s>>>(n, L.d, L.e, L.ranks, cnt,
                                                                                         L.lam);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

// Eigenvectors of the nsel selected eigenvalues (sel: ascending indices into
// L.lam, device; null = all *nw of them) into the first nsel rows of L.Zt.
int ritz_vectors(int n, const RitzLayout& L, const int* sel, int nsel, cudaStream_t s) {
  if (nsel < 1) return SG_OK;
  invit_kernel<<<grid_for((int64_t)nsel * 32, 128), 128, 0, s>>>(n, L.d, L.e, L.ranks, L.lam, sel, nsel, L.Zt, L.lu,
                                                                  L.piv);
  SG_CHECK_LAUNCH();
  constexpr int wpb = 4;
  const size_t sm = (size_t)wpb * n * sizeof(double);
  static_assert(wpb * kRitzMaxN * sizeof(double) <= 48 * 1024, "back-transformation fits default shared memory");
  backtr_kernel<<<(nsel + wpb - 1) / wpb, 32 * wpb, sm, s>>>(n, L.V, L.tau, nsel, L.Zt);
  SG_CHECK_LAUNCH();
  if (nsel > 1) {
    const int64_t pairs = (int64_t)nsel * (nsel + 1) / 2;
    gram_rows_kernel<<<grid_for(pairs * 32, 256), 256, 0, s>>>(nsel, n, L.Zt, L.G);
    SG_CHECK_LAUNCH();
    orth_kernel<<<1, 1024, 0, s>>>(nsel, n, L.G, L.Zt);
    SG_CHECK_LAUNCH();
  }
  return SG_OK;
}

}  // namespace sg

using namespace sg;

extern "C" int64_t sg_sym_eig_work_bytes(int n, int p, int q) {
  if (n < 1 || p < 0 || q < 0 || p + q < 1 || n > kRitzMaxN) return -1;
  const int cnt = p + q >= n ? n : p + q;
  return ritz_layout(nullptr, n, cnt).bytes;
}

extern "C" int sg_sym_eig(int n, const double* A, int64_t lda, int p, int q, double* evals, double* evecs,
                          void* work, int64_t work_bytes, void* stream) {
  if (n < 1 || n > kRitzMaxN || lda < n || !A || !evals || !evecs || !work || p < 0 || q < 0 || p + q < 1)
    return SG_ERR_ARG;
  if (((uintptr_t)work & 255u) != 0) return SG_ERR_ARG;
  const int cnt = p + q >= n ? n : p + q;
  RitzLayout L = ritz_layout((char*)work, n, cnt);
  if (work_bytes < L.bytes) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  int nw = 0;
  int err = ritz_values(n, A, lda, p, q, L, &nw, s);
  if (!err) err = ritz_vectors(n, L, nullptr, nw, s);
  if (err) return err;
  if (cudaMemcpyAsync(evals, L.lam, sizeof(double) * nw, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
      cudaMemcpyAsync(evecs, L.Zt, sizeof(double) * nw * (size_t)n, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
    return SG_ERR_CUDA;
  return SG_OK;
}
