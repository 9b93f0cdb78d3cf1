/*
 * ORACLE -- test infrastructure only.  Tests, the smoke check and the CPU
 * baseline leg of the benchmark compare results with it; the product path
 * never calls it.
 *
 * CPU restatement of the reference's tile binning:
 *   GenomeBaseIndex        snapatac2-core/src/genome.rs:288-406,419-434
 *     new / with_step      genome.rs:296-312, 365-384
 *     get_position_rev     genome.rs:387-406 (panics on pos >= chrom size)
 *     get_position         genome.rs:419-434 (binary search over cumulative
 *                          lengths; panics past the genome end)
 *   FragmentData::get_gindex / exclude   feature_count/data_iter.rs:156-189
 *   gen_mat_pair           feature_count/data_iter.rs:347-415
 *   gen_mat_single         feature_count/data_iter.rs:313-344
 *   to_csr_data            per-row BTreeMap -> sorted (bin, count) rows
 *
 * Every reference panic becomes a status code; the first offending entry
 * (lowest index) is reported through *bad_entry.
 *
 * Build: gcc -O2 -fopenmp -shared -fPIC tile_bin.c -o libtilebin_oracle.so
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_RANGE 2
#define ORC_ERR_CAP 3

/* counting strategies, same meaning as feature_count/counter.rs:19-36 */
#define ORC_INSERTION 0
#define ORC_FRAGMENT 1
#define ORC_PIC 2
#define ORC_SINGLE 3 /* gen_mat_single: +1 at the position's bin */

static int cmp_u64(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return (x > y) - (x < y);
}

typedef struct {
  int n_chrom;
  const uint64_t *base_end; /* cumulative base lengths (genome.rs base_accum_len) */
  const uint8_t *excl;
  uint64_t *bin_off;        /* first output bin of each kept chromosome */
  uint64_t step;
} genome_t;

/* get_position: global base index -> (chrom, offset); -1 past the genome end. */
static int locate(const genome_t *g, uint64_t i, uint64_t *off) {
  int lo = 0, hi = g->n_chrom; /* first c with base_end[c] > i */
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (g->base_end[mid] <= i) lo = mid + 1; else hi = mid;
  }
  if (lo >= g->n_chrom) return -1;
  *off = i - (lo ? g->base_end[lo - 1] : 0);
  return lo;
}

static uint64_t chrom_size(const genome_t *g, int c) {
  return g->base_end[c] - (c ? g->base_end[c - 1] : 0);
}

/* Collect the bins hit by one row (unsorted, with repeats).  Returns the
 * number of keys, or a negative value with *err set. */
static int64_t row_keys(const genome_t *g, const uint64_t *pos, const uint32_t *len,
                        int64_t a, int64_t b, int strategy, int64_t min_len, int64_t max_len,
                        uint64_t **buf, int64_t *bufcap, int *err, int64_t *bad) {
  int64_t nk = 0;
  for (int64_t k = a; k < b; ++k) {
    uint64_t start;
    int c = locate(g, pos[k], &start);
    if (c < 0) { *err = ORC_ERR_RANGE; *bad = k; return -1; }
    uint64_t lo_bin, hi_bin;
    int emit2 = 0;
    if (strategy == ORC_SINGLE) {
      if (g->excl[c]) continue;
      lo_bin = hi_bin = g->bin_off[c] + start / g->step;
    } else {
      uint64_t fs = (uint64_t)len[k];
      uint64_t end = start + fs - 1; /* u64 arithmetic, wraps like the reference */
      if (g->excl[c]) continue;
      if (min_len >= 0 && fs < (uint64_t)min_len) continue;
      if (max_len >= 0 && fs > (uint64_t)max_len) continue;
      uint64_t sz = chrom_size(g, c);
      if (end >= sz) { *err = ORC_ERR_RANGE; *bad = k; return -1; }
      lo_bin = g->bin_off[c] + start / g->step;
      hi_bin = g->bin_off[c] + end / g->step;
      if (strategy == ORC_INSERTION) emit2 = 1;
    }
    int64_t need;
    if (strategy == ORC_FRAGMENT) need = hi_bin >= lo_bin ? (int64_t)(hi_bin - lo_bin + 1) : 0;
    else if (strategy == ORC_PIC) need = (hi_bin != lo_bin) ? 2 : 1;
    else if (strategy == ORC_INSERTION) need = 2;
    else need = 1;
    if (nk + need > *bufcap) {
      int64_t nc = (*bufcap * 2 > nk + need) ? *bufcap * 2 : nk + need + 64;
      uint64_t *nb = (uint64_t *)realloc(*buf, (size_t)nc * sizeof(uint64_t));
      if (!nb) { *err = ORC_ERR_ARG; return -1; }
      *buf = nb; *bufcap = nc;
    }
    uint64_t *o = *buf + nk;
    if (strategy == ORC_FRAGMENT) {
      for (uint64_t x = lo_bin; x <= hi_bin && hi_bin >= lo_bin; ++x) *o++ = x;
    } else if (strategy == ORC_PIC) {
      *o++ = lo_bin;
      if (hi_bin != lo_bin) *o++ = hi_bin;
    } else if (emit2) {
      *o++ = lo_bin; *o++ = hi_bin;
    } else {
      *o++ = lo_bin;
    }
    nk += need;
  }
  return nk;
}

/*
 * Bin fragments of every cell.  Pass out_idx == NULL to only count: then
 * out_indptr[0..n_cells] receives the CSR row pointer and the return value
 * is nnz.  With out_idx/out_cnt given (capacity cap) the rows are filled.
 * chrom_len: per-chromosome base length (all >= 1); chrom_excl: 1 = dropped.
 * min_len/max_len: -1 = no bound.  Returns nnz (>= 0) or -status.
 */
int64_t oracle_tile_bin(const int64_t *cell_ptr, int64_t n_cells, const uint64_t *pos,
                        const uint32_t *len, const uint64_t *chrom_len, const uint8_t *chrom_excl,
                        int n_chrom, uint64_t bin_size, int strategy, int64_t min_len,
                        int64_t max_len, int64_t *out_indptr, int32_t *out_idx, uint32_t *out_cnt,
                        int64_t cap, int64_t *bad_entry) {
  if (n_chrom <= 0 || bin_size == 0 || strategy < 0 || strategy > 3 || n_cells < 0) return -ORC_ERR_ARG;
  uint64_t *base_end = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n_chrom);
  uint64_t *bin_off = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)n_chrom);
  uint64_t acc = 0, bacc = 0;
  for (int c = 0; c < n_chrom; ++c) {
    if (chrom_len[c] == 0) { free(base_end); free(bin_off); return -ORC_ERR_ARG; }
    acc += chrom_len[c];
    base_end[c] = acc;
    bin_off[c] = bacc;
    if (!chrom_excl[c]) bacc += (chrom_len[c] + bin_size - 1) / bin_size;
  }
  genome_t g = {n_chrom, base_end, chrom_excl, bin_off, bin_size};
  int err = ORC_OK;
  int64_t bad = INT64_MAX;
  int fill = out_idx != NULL;
  if (!fill) out_indptr[0] = 0;

#pragma omp parallel
  {
    uint64_t *buf = NULL;
    int64_t bufcap = 0;
    int lerr = ORC_OK;
    int64_t lbad = INT64_MAX;
#pragma omp for schedule(dynamic, 16)
    for (int64_t r = 0; r < n_cells; ++r) {
      int e = ORC_OK;
      int64_t b = INT64_MAX;
      int64_t nk = row_keys(&g, pos, len, cell_ptr[r], cell_ptr[r + 1], strategy, min_len, max_len,
                            &buf, &bufcap, &e, &b);
      if (nk < 0) {
        if (lerr == ORC_OK || b < lbad) { lerr = e; lbad = b; }
        continue;
      }
      qsort(buf, (size_t)nk, sizeof(uint64_t), cmp_u64);
      int64_t nu = 0;
      if (fill) {
        int64_t o = out_indptr[r];
        int64_t lim = out_indptr[r + 1];
        for (int64_t i = 0; i < nk;) {
          int64_t j = i;
          while (j < nk && buf[j] == buf[i]) ++j;
          if (o + nu < lim && o + nu < cap) {
            out_idx[o + nu] = (int32_t)buf[i];
            out_cnt[o + nu] = (uint32_t)(j - i);
          }
          ++nu;
          i = j;
        }
      } else {
        for (int64_t i = 0; i < nk; ++i) if (i == 0 || buf[i] != buf[i - 1]) ++nu;
        out_indptr[r + 1] = nu;
      }
    }
    free(buf);
#pragma omp critical
    {
      if (lerr != ORC_OK && (err == ORC_OK || lbad < bad)) { err = lerr; bad = lbad; }
    }
  }
  free(base_end);
  free(bin_off);
  if (err != ORC_OK) {
    if (bad_entry) *bad_entry = bad;
    return -err;
  }
  if (!fill) {
    for (int64_t r = 0; r < n_cells; ++r) out_indptr[r + 1] += out_indptr[r];
    return out_indptr[n_cells];
  }
  if (out_indptr[n_cells] > cap) return -ORC_ERR_CAP;
  return out_indptr[n_cells];
}

/* Number of output columns: sum over kept chromosomes of ceil(len / bin). */
uint64_t oracle_tile_ncols(const uint64_t *chrom_len, const uint8_t *chrom_excl, int n_chrom,
                           uint64_t bin_size) {
  uint64_t t = 0;
  for (int c = 0; c < n_chrom; ++c)
    if (!chrom_excl[c]) t += (chrom_len[c] + bin_size - 1) / bin_size;
  return t;
}
