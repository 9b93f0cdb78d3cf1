/*
 * ORACLE -- test infrastructure only (tests and the CPU legs of the bench).
 *
 * The matvec of the reference's eigensolve, restating
 *   snapatac2-python/src/embedding.rs:155-171  eigen: the LinearOperator
 *     f(v) = X @ (v.T @ X).T - D * v   (X the degree-scaled CSR, D = 1/(d-1))
 * in FP64 with OpenMP: t = X^T v over the CSC (one column per iteration,
 * rows ascending), then out = X t - D v over the CSR (one row per
 * iteration, columns ascending).  SciPy's CSR products run single-threaded
 * with another summation order; the sums are the same to FP64 rounding, so
 * eigsh converges to the same eigenpairs.  This only shortens the oracle's
 * wall time at sizes where SciPy's matvec would take minutes.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC gram.c -o libgram_oracle.so
 */
#include <stdint.h>

int oracle_gram_matvec(int64_t n, int64_t m, const int64_t *indptr, const int32_t *indices, const double *data,
                       const int64_t *colptr, const int32_t *rowidx, const double *cdata, const double *D,
                       const double *v, double *t, double *out) {
  if (n <= 0 || m <= 0) return 1;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t j = 0; j < m; ++j) {
    double s = 0.0;
    for (int64_t e = colptr[j]; e < colptr[j + 1]; ++e) s += cdata[e] * v[rowidx[e]];
    t[j] = s;
  }
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    double s = 0.0;
    for (int64_t e = indptr[i]; e < indptr[i + 1]; ++e) s += data[e] * t[indices[e]];
    out[i] = s - D[i] * v[i];
  }
  return 0;
}
