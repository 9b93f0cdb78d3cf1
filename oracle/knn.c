/*
 * ORACLE -- test infrastructure only (tests and the CPU-baseline leg).
 *
 * Exact Euclidean k-nearest-neighbour graph, restating
 *   snapatac2-core/src/utils/knn.rs:9-31  nearest_neighbour_graph
 *     kd-tree iter_nearest with squared_euclidean (kdtree 0.7 crate), self
 *     removed by index (not by distance), first k kept, value = sqrt(dist)
 *   snapatac2-core/src/utils/knn.rs:58-78  to_csr_matrix: each row sorted
 *     by column index.
 * The kd-tree only orders candidates; the k nearest set is unique up to
 * exact distance ties, so a brute-force scan in FP64 with the same
 * sum((a-b)^2) arithmetic is an equivalent oracle.  Ties are broken by the
 * smaller point index.
 *
 * Build: gcc -O2 -fopenmp -shared -fPIC knn.c -o libknn_oracle.so
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

typedef struct {
  double d;
  int64_t j;
} cand_t;

static int worse(const cand_t *a, const cand_t *b) { /* a ranks after b */
  return a->d > b->d || (a->d == b->d && a->j > b->j);
}

/* max-heap of the k best so far, root = worst kept candidate */
static void sift_down(cand_t *h, int k, int i) {
  for (;;) {
    int l = 2 * i + 1, r = l + 1, m = i;
    if (l < k && worse(&h[l], &h[m])) m = l;
    if (r < k && worse(&h[r], &h[m])) m = r;
    if (m == i) return;
    cand_t t = h[i]; h[i] = h[m]; h[m] = t;
    i = m;
  }
}

static int cmp_idx(const void *a, const void *b) {
  int64_t x = ((const cand_t *)a)->j, y = ((const cand_t *)b)->j;
  return (x > y) - (x < y);
}

/*
 * X: row-major n x d doubles.  Queries q0..q1-1 (all points are candidates).
 * Output rows (q - q0) of nbr/dist (k entries each), sorted by column index,
 * dist = sqrt(squared distance).  Needs k <= n - 1.  Returns 0 or -1.
 */
int oracle_knn(const double *X, int64_t n, int d, int k, int64_t q0, int64_t q1, int64_t *nbr,
               double *dist) {
  if (k <= 0 || k > n - 1 || q0 < 0 || q1 > n || q0 > q1) return -1;
#pragma omp parallel
  {
    cand_t *h = (cand_t *)malloc(sizeof(cand_t) * (size_t)k);
#pragma omp for schedule(dynamic, 8)
    for (int64_t q = q0; q < q1; ++q) {
      const double *x = X + q * (int64_t)d;
      int cnt = 0;
      for (int64_t j = 0; j < n; ++j) {
        if (j == q) continue;
        const double *y = X + j * (int64_t)d;
        double s = 0.0;
        for (int t = 0; t < d; ++t) {
          double u = x[t] - y[t];
          s += u * u;
        }
        cand_t c = {s, j};
        if (cnt < k) {
          h[cnt++] = c;
          if (cnt == k)
            for (int i = k / 2 - 1; i >= 0; --i) sift_down(h, k, i);
        } else if (worse(&h[0], &c)) {
          h[0] = c;
          sift_down(h, k, 0);
        }
      }
      qsort(h, (size_t)k, sizeof(cand_t), cmp_idx);
      int64_t o = (q - q0) * (int64_t)k;
      for (int i = 0; i < k; ++i) {
        nbr[o + i] = h[i].j;
        dist[o + i] = sqrt(h[i].d);
      }
    }
    free(h);
  }
  return 0;
}
