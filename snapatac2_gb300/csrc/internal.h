// Internal (C++ linkage) helpers shared between translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace sg {

constexpr int kScanBlock = 512;
constexpr int kScanItems = 8;
constexpr int64_t kScanTile = (int64_t)kScanBlock * kScanItems;

// In-place inclusive prefix sum of n int64 values.  `scratch` needs
// scan_scratch_bytes(n) bytes.  Deterministic.
cudaError_t inclusive_scan_i64(int64_t* data, int64_t n, void* scratch, cudaStream_t s);
int64_t scan_scratch_bytes(int64_t n);

// Stable LSD radix sort of n 64-bit keys (and 64-bit payloads when vals is
// not null) by key bits [begin_bit, end_bit), 8 bits per pass, ping-ponging
// between (keys, vals) and (keys_alt, vals_alt); *in_alt tells which pair
// holds the result.  `scratch` needs radix_scratch_bytes(n) bytes.
cudaError_t radix_sort_u64(int64_t n, uint64_t* keys, uint64_t* vals, uint64_t* keys_alt, uint64_t* vals_alt,
                           int begin_bit, int end_bit, void* scratch, cudaStream_t s, bool* in_alt);
int64_t radix_scratch_bytes(int64_t n);

// Dense symmetric FP64 eigensolver of the Rayleigh-Ritz step (ritz.cu).
constexpr int kRitzMaxN = 640;  // largest matrix the cluster reduction holds in shared memory

struct RitzLayout {
  double* d;           // tridiagonal: diagonal
  double* e;           //              off-diagonal
  double* tau;         // Householder scalars
  double* V;           // n x n, row j = reflector j
  int* ranks;          // ascending ranks of the wanted eigenvalues
  double* lam;         // their values, ascending
  double* Zt;          // eigenvectors of the selected ones (rows)
  double* lu;          // inverse-iteration scratch
  unsigned char* piv;  //
  double* G;           // Gram matrix of the selected vectors (Cholesky-QR)
  int64_t bytes;
};
RitzLayout ritz_layout(char* base, int n, int nw);
int ritz_values(int n, const double* A, int64_t lda, int p, int q, const RitzLayout& L, int* nw, cudaStream_t s);
int ritz_vectors(int n, const RitzLayout& L, const int* sel, int nsel, cudaStream_t s);
int ritz_cluster_size(int n);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

inline int grid_for(int64_t n, int block, int max_blocks = 1 << 20) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

}  // namespace sg
