/*
 * ORACLE -- test infrastructure only.  Tests and the CPU baseline leg of the
 * benchmark compare results with it; the product path never calls it.
 *
 * Cell-by-region counts (the peak matrix over fragments) restated in C for
 * a compiled-speed CPU baseline; oracle/regions.py holds the loop-for-loop
 * Python restatement this file is tested against.
 *   create_peak_matrix       snapatac2-core/src/feature_count/matrix.rs:95-170
 *   pair_to_fragments /      feature_count/data_iter.rs:27-117: paired rows
 *   single_to_fragments      give [start, start + size) after the size
 *                            filters, single-end rows a 1 bp read
 *   RegionCounter::insert_fragment  feature_count/counter.rs:117-146:
 *     insertion   +1 per region overlapping each insertion ([s, s + 1) and
 *                 [e - 1, e)); a region hit by both gets 2
 *     fragment    +1 per region overlapping [s, e)
 *     paired-insertion  +1 once per region hit by either insertion
 *     single      +1 per region overlapping the 1 bp read
 * Regions are the caller's, per chromosome sorted by start with the running
 * maximum of the ends (an interval index): a query [qs, qe) hits region i
 * when start_i < qe and end_i > qs.  Row entries sorted by region id.
 *
 * Two calls: pass 0 writes each cell's entry count to out_ptr[r + 1]; the
 * caller turns out_ptr into offsets; pass 1 writes out_idx / out_val.
 * Cells run in parallel (OpenMP, dynamic schedule); results do not depend
 * on the thread count.  A position at or past the genome end gives
 * ORC_ERR_RANGE with the lowest offending fragment in *bad.
 *
 * Build: gcc -O2 -fopenmp -shared -fPIC regions.c -o libregions_oracle.so
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_RANGE 2

#define ORC_INSERTION 0
#define ORC_FRAGMENT 1
#define ORC_PIC 2
#define ORC_SINGLE 3

typedef struct {
  int64_t *v;
  int64_t n, cap;
} Vec;

static int vec_push(Vec *a, int64_t x) {
  if (a->n == a->cap) {
    int64_t c = a->cap ? 2 * a->cap : 256;
    int64_t *p = (int64_t *)realloc(a->v, (size_t)c * sizeof(int64_t));
    if (!p) return -1;
    a->v = p;
    a->cap = c;
  }
  a->v[a->n++] = x;
  return 0;
}

static int cmp_i64(const void *a, const void *b) {
  int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

typedef struct {
  const int64_t *ptr, *start, *end, *maxend, *id;
} Regions;

/* region ids of chromosome c overlapping [qs, qe), appended to out */
static int hits(const Regions *R, int c, int64_t qs, int64_t qe, Vec *out) {
  int64_t lo = R->ptr[c], hi = R->ptr[c + 1];
  /* first region whose start is >= qe */
  int64_t a = lo, b = hi;
  while (a < b) {
    int64_t m = a + (b - a) / 2;
    if (R->start[m] < qe) a = m + 1;
    else b = m;
  }
  for (int64_t i = a - 1; i >= lo; --i) {
    if (R->maxend[i] <= qs) break;
    if (R->end[i] > qs && vec_push(out, R->id[i])) return -1;
  }
  return 0;
}

static int in_list(const int64_t *v, int64_t n, int64_t x) {
  for (int64_t i = 0; i < n; ++i)
    if (v[i] == x) return 1;
  return 0;
}

int oracle_region_counts(int pass, int64_t n_cells, const int64_t *indptr, const uint64_t *pos, const uint32_t *len,
                         int n_chrom, const uint64_t *chrom_start, const int64_t *rptr, const int64_t *rstart,
                         const int64_t *rend, const int64_t *rmaxend, const int64_t *rid, int strategy,
                         int64_t min_len, int64_t max_len, int n_threads, int64_t *out_ptr, int64_t *out_idx,
                         uint32_t *out_val, int64_t *bad) {
  if (n_cells < 0 || n_chrom < 1 || strategy < 0 || strategy > 3 || (strategy != ORC_SINGLE && !len)) return ORC_ERR_ARG;
  const Regions R = {rptr, rstart, rend, rmaxend, rid};
  const uint64_t genome = chrom_start[n_chrom];
  int err = ORC_OK;
  int64_t first_bad = INT64_MAX;
#ifdef _OPENMP
  const int nt = n_threads > 0 ? n_threads : omp_get_max_threads();
#else
  (void)n_threads;
#endif
#pragma omp parallel num_threads(nt)
  {
    Vec h = {0, 0, 0}, q1 = {0, 0, 0}, q2 = {0, 0, 0};
    int local_err = ORC_OK;
    int64_t local_bad = INT64_MAX;
#pragma omp for schedule(dynamic, 16)
    for (int64_t r = 0; r < n_cells; ++r) {
      h.n = 0;
      for (int64_t j = indptr[r]; j < indptr[r + 1] && !local_err; ++j) {
        const uint64_t p = pos[j];
        if (p >= genome) {
          if (j < local_bad) local_bad = j;
          break;  /* this cell's row is abandoned; the call reports the error */
        }
        int a = 0, b = n_chrom; /* chromosome: last start <= p */
        while (b - a > 1) {
          int m = (a + b) / 2;
          if (chrom_start[m] <= p) a = m;
          else b = m;
        }
        const int64_t s = (int64_t)(p - chrom_start[a]);
        int rc = 0;
        if (strategy == ORC_SINGLE) {
          rc = hits(&R, a, s, s + 1, &h);
        } else {
          const int64_t size = (int64_t)len[j];
          if (min_len >= 0 && size < min_len) continue;
          if (max_len >= 0 && size > max_len) continue;
          const int64_t e = s + size;
          if (strategy == ORC_FRAGMENT) {
            rc = hits(&R, a, s, e, &h);
          } else if (strategy == ORC_INSERTION) {
            rc = hits(&R, a, s, s + 1, &h) || hits(&R, a, e - 1, e, &h);
          } else {
            q1.n = q2.n = 0;
            rc = hits(&R, a, s, s + 1, &q1) || hits(&R, a, e - 1, e, &q2);
            for (int64_t i = 0; !rc && i < q1.n; ++i)
              if (!in_list(q1.v, i, q1.v[i])) rc = vec_push(&h, q1.v[i]);
            for (int64_t i = 0; !rc && i < q2.n; ++i)
              if (!in_list(q1.v, q1.n, q2.v[i]) && !in_list(q2.v, i, q2.v[i])) rc = vec_push(&h, q2.v[i]);
          }
        }
        if (rc) local_err = ORC_ERR_ARG; /* out of memory */
      }
      if (h.n > 1) qsort(h.v, (size_t)h.n, sizeof(int64_t), cmp_i64);
      int64_t k = 0, o = pass == 1 ? out_ptr[r] : 0;
      for (int64_t i = 0; i < h.n;) {
        int64_t j = i;
        while (j < h.n && h.v[j] == h.v[i]) ++j;
        if (pass == 1) {
          out_idx[o + k] = h.v[i];
          out_val[o + k] = (uint32_t)(j - i);
        }
        ++k;
        i = j;
      }
      if (pass == 0) out_ptr[r + 1] = k;
    }
#pragma omp critical
    {
      if (local_err && !err) err = local_err;
      if (local_bad < first_bad) first_bad = local_bad;
    }
    free(h.v);
    free(q1.v);
    free(q2.v);
  }
  if (err) return err;
  if (first_bad != INT64_MAX) {
    if (bad) *bad = first_bad;
    return ORC_ERR_RANGE;
  }
  if (pass == 0) out_ptr[0] = 0;
  return ORC_OK;
}
