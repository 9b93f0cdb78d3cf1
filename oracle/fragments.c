/*
 * ORACLE (test infrastructure only): the fragment-file import restated in C.
 *
 * Same algorithm as oracle/fragments.py (record syntax of
 * snapatac2-core/src/preprocessing/qc.rs:303-348, shifts of
 * snapatac2-python/src/preprocessing.rs:174-184, the unsorted-input
 * whitelist and sort of preprocessing.rs:106-152, grouping, QC, filters and
 * per-cell sort of snapatac2-core/src/preprocessing/import.rs:31-210), in
 * compiled code so that a CPU baseline of realistic speed can be timed.  One
 * thread; qsort for the sorts.  Results are returned in malloc'd arrays that
 * the caller frees with oracle_import_free.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

enum { E_OK = 0, E_PARSE = 7, E_UNSORTED = 8, E_RANGE = 2, E_CONVERT = 9 };

typedef struct {
  int64_t bc_off;   /* -1: no barcode (".") */
  int32_t bc_len;
  int32_t chrom;    /* index into the sorted names, -1: not in the genome */
  uint64_t start, end;
  uint32_t count;
  int8_t strand;    /* 0 none, 1 "+", 2 "-" */
  int64_t line;
} Rec;

typedef struct {
  int64_t n_cells, nnz, paired, bad_line, error;
  int64_t* indptr;
  int64_t* indices;
  int64_t* data;          /* signed sizes (uint32 or int32 range) */
  int64_t* bc_off;        /* per cell: barcode location in the text */
  int32_t* bc_len;
  uint64_t* n_fragment;
  double* frac_dup;
  double* frac_mito;
} ImportOut;

static const char* g_text;

static int cmp_bytes(const char* a, int64_t na, const char* b, int64_t nb) {
  const int64_t m = na < nb ? na : nb;
  const int c = memcmp(a, b, (size_t)m);
  if (c) return c < 0 ? -1 : 1;
  return na < nb ? -1 : (na > nb ? 1 : 0);
}

static int parse_uint(const char* p, int64_t n, int bits, uint64_t* out) {
  if (n <= 0) return 0;
  uint64_t v = 0;
  for (int64_t i = 0; i < n; ++i) {
    const unsigned d = (unsigned)(unsigned char)p[i] - '0';
    if (d > 9) return 0;
    if (v > (UINT64_MAX - d) / 10) return 0;
    v = v * 10 + d;
  }
  if (bits < 64 && (v >> bits)) return 0;
  *out = v;
  return 1;
}

static uint64_t sat_add(uint64_t x, int64_t s) {
  if (s >= 0) return x > UINT64_MAX - (uint64_t)s ? UINT64_MAX : x + (uint64_t)s;
  const uint64_t m = (uint64_t)(-(s + 1)) + 1;
  return x < m ? 0 : x - m;
}

/* binary search over names sorted by bytes */
static int find_name(const char* blob, const int64_t* off, int n, const char* q, int64_t ql) {
  int lo = 0, hi = n - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) / 2;
    const int c = cmp_bytes(q, ql, blob + off[mid], off[mid + 1] - off[mid]);
    if (!c) return mid;
    if (c < 0) hi = mid - 1;
    else lo = mid + 1;
  }
  return -1;
}

static const Rec* g_recs;
static int cmp_rec_bc(const void* a, const void* b) {  /* barcode bytes ("." first), then line */
  const Rec* x = &g_recs[*(const int64_t*)a];
  const Rec* y = &g_recs[*(const int64_t*)b];
  if ((x->bc_off < 0) != (y->bc_off < 0)) return x->bc_off < 0 ? -1 : 1;
  if (x->bc_off >= 0) {
    const int c = cmp_bytes(g_text + x->bc_off, x->bc_len, g_text + y->bc_off, y->bc_len);
    if (c) return c;
  }
  return x->line < y->line ? -1 : (x->line > y->line ? 1 : 0);
}

typedef struct { int64_t pos, val; } PV;
static int cmp_pv(const void* a, const void* b) {
  const PV* x = (const PV*)a;
  const PV* y = (const PV*)b;
  if (x->pos != y->pos) return x->pos < y->pos ? -1 : 1;
  return x->val < y->val ? -1 : (x->val > y->val ? 1 : 0);
}

static int same_bc(const Rec* a, const Rec* b) {
  return a->bc_len == b->bc_len && !memcmp(g_text + a->bc_off, g_text + b->bc_off, (size_t)a->bc_len);
}

typedef struct { int64_t off; int32_t len; } Str;
static int cmp_str(const void* a, const void* b) {
  const Str* x = (const Str*)a;
  const Str* y = (const Str*)b;
  return cmp_bytes(g_text + x->off, x->len, g_text + y->off, y->len);
}

static const char* g_wl;
static const int64_t* g_wl_off;
static int64_t g_wl_n;
static int in_whitelist(const char* q, int64_t ql) {  /* whitelist sorted by bytes */
  int64_t lo = 0, hi = g_wl_n - 1;
  while (lo <= hi) {
    const int64_t mid = (lo + hi) / 2;
    const int c = cmp_bytes(q, ql, g_wl + g_wl_off[mid], g_wl_off[mid + 1] - g_wl_off[mid]);
    if (!c) return 1;
    if (c < 0) hi = mid - 1;
    else lo = mid + 1;
  }
  return 0;
}

void oracle_import_free(ImportOut* o) {
  free(o->indptr); free(o->indices); free(o->data); free(o->bc_off); free(o->bc_len);
  free(o->n_fragment); free(o->frac_dup); free(o->frac_mito);
  memset(o, 0, sizeof(*o));
}

#define FAIL(code, ln) do { out->error = (code); out->bad_line = (ln); goto done; } while (0)

int64_t oracle_import(const char* text, int64_t nbytes, const char* cblob, const int64_t* coff, const uint64_t* csize,
                      const uint64_t* cbase, const uint8_t* cmito, int n_chrom, const char* wl, const int64_t* wl_off,
                      int64_t n_wl, int has_wl, uint64_t min_frag, int sorted_input, int64_t shift_left,
                      int64_t shift_right, ImportOut* out) {
  memset(out, 0, sizeof(*out));
  out->bad_line = -1;
  out->paired = -1;
  g_text = text;
  g_wl = wl; g_wl_off = wl_off; g_wl_n = n_wl;
  int64_t cap = 1024, nrec = 0;
  Rec* recs = (Rec*)malloc(sizeof(Rec) * cap);
  int64_t* order = NULL;
  int64_t* gstart = NULL;
  uint8_t* pre_ok = NULL;
  PV* pv = NULL;
  int64_t *cells_ptr = NULL, *cells_idx = NULL, *cells_val = NULL;
  /* lines */
  int64_t line = 0;
  for (int64_t s = 0; s < nbytes || (s == nbytes && 0); ++line) {
    const char* nlp = memchr(text + s, '\n', (size_t)(nbytes - s));
    int64_t e = nlp ? (int64_t)(nlp - text) : nbytes;
    const int64_t next = nlp ? e + 1 : nbytes + 1;
    if (nlp && e > s && text[e - 1] == '\r') --e;
    if (e > s && text[s] == '#') { s = next; continue; }
    int64_t fs[6], fe[6];
    int nf = 0;
    int64_t a = s;
    for (int64_t p = s;; ++p) {
      if (p == e || text[p] == '\t') {
        fs[nf] = a; fe[nf] = p; ++nf; a = p + 1;
        if (p == e || nf == 6) break;
      }
    }
    Rec r;
    memset(&r, 0, sizeof(r));
    r.line = line;
    uint64_t cnt = 1;
    int ok = nf >= 4 && parse_uint(text + fs[1], fe[1] - fs[1], 64, &r.start) &&
             parse_uint(text + fs[2], fe[2] - fs[2], 64, &r.end);
    if (ok && nf >= 5 && !(fe[4] - fs[4] == 1 && text[fs[4]] == '.')) ok = parse_uint(text + fs[4], fe[4] - fs[4], 32, &cnt);
    if (ok && nf >= 6) {
      const int64_t n = fe[5] - fs[5];
      const char c = n == 1 ? text[fs[5]] : 0;
      if (c == '+') r.strand = 1;
      else if (c == '-') r.strand = 2;
      else if (c != '.') ok = 0;
    }
    if (!ok) { free(recs); out->error = E_PARSE; out->bad_line = line; return E_PARSE; }
    r.count = (uint32_t)cnt;
    const int64_t bl = fe[3] - fs[3];
    if (bl == 1 && text[fs[3]] == '.') r.bc_off = -1;
    else { r.bc_off = fs[3]; r.bc_len = (int32_t)bl; }
    r.chrom = find_name(cblob, coff, n_chrom, text + fs[0], fe[0] - fs[0]);
    if (shift_left) {
      r.start = sat_add(r.start, shift_left);
      if (r.strand) r.end = sat_add(r.end, shift_left);
    }
    if (shift_right && !r.strand) r.end = sat_add(r.end, shift_right);
    if (nrec == cap) { cap *= 2; recs = (Rec*)realloc(recs, sizeof(Rec) * cap); }
    recs[nrec++] = r;
    s = next;
  }
  g_recs = recs;
  if (nrec == 0) { free(recs); return E_OK; }
  out->paired = recs[0].strand == 0;
  const int paired = (int)out->paired;
  order = (int64_t*)malloc(sizeof(int64_t) * nrec);
  for (int64_t i = 0; i < nrec; ++i) order[i] = i;
  const int pre = !sorted_input && min_frag > 0;
  if (pre)
    for (int64_t i = 0; i < nrec; ++i)
      if (recs[i].bc_off < 0) FAIL(E_PARSE, recs[i].line);
  if (!sorted_input) qsort(order, (size_t)nrec, sizeof(int64_t), cmp_rec_bc);
  /* records kept for grouping: end != start, in `order` */
  int64_t nk = 0;
  for (int64_t i = 0; i < nrec; ++i) {
    const Rec* r = &recs[order[i]];
    if (r->end == r->start) continue;
    if (r->bc_off < 0) FAIL(E_PARSE, r->line);
    order[nk++] = order[i];
  }
  /* minimum-count whitelist of unsorted input: all records of the barcode */
  if (pre) {
    /* count all records per barcode: the sorted order of all records is contiguous per barcode */
    int64_t* all = (int64_t*)malloc(sizeof(int64_t) * nrec);
    for (int64_t i = 0; i < nrec; ++i) all[i] = i;
    qsort(all, (size_t)nrec, sizeof(int64_t), cmp_rec_bc);
    pre_ok = (uint8_t*)calloc((size_t)nrec, 1);  /* per record: its barcode passes */
    for (int64_t a = 0; a < nrec;) {
      int64_t b = a + 1;
      while (b < nrec && same_bc(&recs[all[a]], &recs[all[b]])) ++b;
      const uint8_t ok2 = (uint64_t)(b - a) >= min_frag;
      for (int64_t j = a; j < b; ++j) pre_ok[all[j]] = ok2;
      a = b;
    }
    free(all);
  }
  /* groups: runs of equal barcode */
  gstart = (int64_t*)malloc(sizeof(int64_t) * (nk + 1));
  int64_t ng = 0;
  for (int64_t i = 0; i < nk; ++i)
    if (i == 0 || !same_bc(&recs[order[i]], &recs[order[i - 1]])) gstart[ng++] = i;
  gstart[ng] = nk;
  /* processed groups and the sorted-input check */
  {
    Str* seen = (Str*)malloc(sizeof(Str) * (ng + 1));
    int64_t ns = 0;
    uint8_t* proc = (uint8_t*)calloc((size_t)ng + 1, 1);
    for (int64_t g = 0; g < ng; ++g) {
      const Rec* r0 = &recs[order[gstart[g]]];
      int ok2 = !has_wl || in_whitelist(text + r0->bc_off, r0->bc_len);
      if (pre) ok2 = ok2 && pre_ok[order[gstart[g]]];
      proc[g] = (uint8_t)ok2;
      if (ok2) { seen[ns].off = r0->bc_off; seen[ns].len = r0->bc_len; ++ns; }
    }
    qsort(seen, (size_t)ns, sizeof(Str), cmp_str);
    for (int64_t i = 1; i < ns; ++i)
      if (!cmp_str(&seen[i - 1], &seen[i])) { free(seen); free(proc); FAIL(E_UNSORTED, -1); }
    free(seen);
    /* per processed group: QC, values, errors */
    cells_ptr = (int64_t*)malloc(sizeof(int64_t) * (ng + 1));
    cells_idx = (int64_t*)malloc(sizeof(int64_t) * (nk + 1));
    cells_val = (int64_t*)malloc(sizeof(int64_t) * (nk + 1));
    out->bc_off = (int64_t*)malloc(sizeof(int64_t) * (ng + 1));
    out->bc_len = (int32_t*)malloc(sizeof(int32_t) * (ng + 1));
    out->n_fragment = (uint64_t*)malloc(sizeof(uint64_t) * (ng + 1));
    out->frac_dup = (double*)malloc(sizeof(double) * (ng + 1));
    out->frac_mito = (double*)malloc(sizeof(double) * (ng + 1));
    pv = (PV*)malloc(sizeof(PV) * (nk + 1));
    int64_t nc = 0, nz = 0;
    cells_ptr[0] = 0;
    for (int64_t g = 0; g < ng; ++g) {
      if (!proc[g]) continue;
      uint64_t uniq = 0, mito = 0, total = 0;
      int64_t np = 0;
      for (int64_t j = gstart[g]; j < gstart[g + 1]; ++j) {
        const Rec* r = &recs[order[j]];
        if (r->chrom < 0) continue;
        total += r->count;
        if (cmito[r->chrom]) ++mito;
        else ++uniq;
        const int64_t si = (int64_t)r->start, ei = (int64_t)r->end;
        const int64_t size = (int64_t)((uint64_t)ei - (uint64_t)si);
        uint64_t p;
        int64_t v;
        if (r->strand == 2) { p = (uint64_t)ei - 1u; v = (int64_t)(0u - (uint64_t)size); }
        else { p = r->start; v = size; }
        if (p >= csize[r->chrom]) { free(proc); FAIL(E_RANGE, r->line); }
        if (paired ? !(v >= 0 && v <= (int64_t)UINT32_MAX) : !(v >= INT32_MIN && v <= INT32_MAX)) {
          free(proc);
          FAIL(E_CONVERT, r->line);
        }
        pv[np].pos = (int64_t)(cbase[r->chrom] + p);
        pv[np].val = v;
        ++np;
      }
      if (uniq < min_frag) continue;
      qsort(pv, (size_t)np, sizeof(PV), cmp_pv);
      for (int64_t j = 0; j < np; ++j) { cells_idx[nz] = pv[j].pos; cells_val[nz] = pv[j].val; ++nz; }
      const Rec* r0 = &recs[order[gstart[g]]];
      out->bc_off[nc] = r0->bc_off;
      out->bc_len[nc] = r0->bc_len;
      out->n_fragment[nc] = uniq;
      out->frac_dup[nc] = 1.0 - (double)(uniq + mito) / (double)total;
      out->frac_mito[nc] = (double)mito / (double)(uniq + mito);
      ++nc;
      cells_ptr[nc] = nz;
    }
    free(proc);
    out->n_cells = nc;
    out->nnz = nz;
    out->indptr = cells_ptr; cells_ptr = NULL;
    out->indices = cells_idx; cells_idx = NULL;
    out->data = cells_val; cells_val = NULL;
  }
done:
  free(recs); free(order); free(gstart); free(pre_ok); free(pv);
  free(cells_ptr); free(cells_idx); free(cells_val);
  if (out->error) {
    const int64_t e = out->error, bl = out->bad_line, pr = out->paired;
    oracle_import_free(out);
    out->error = e; out->bad_line = bl; out->paired = pr;
  }
  return out->error;
}
