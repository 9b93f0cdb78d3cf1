/*
 * snapgb300 -- C ABI of the GB300 kernels behind the SnapATAC2-compatible
 * cell-embedding path (tile binning, matrix-free cosine spectral embedding,
 * exact kNN).
 *
 * Conventions
 *  - Every entry point returns an int status: SG_OK (0) or one of SG_ERR_*.
 *    No exceptions cross the ABI.
 *  - All array arguments are DEVICE pointers owned by the caller unless the
 *    comment says "host".  The library allocates nothing on the device.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *    Every call only enqueues work on that stream; results are ready after
 *    the stream is synchronised.
 *  - Data-dependent failures (a fragment past the end of its chromosome, an
 *    output buffer that is too small) are reported through a device-side
 *    status word `status` (int, set to the first SG_ERR_* seen, 0 otherwise)
 *    and `bad` (uint64, lowest offending input index), which the caller reads
 *    after synchronising.  The reference raises a Rust panic in those cases.
 *  - Entry points are re-entrant per stream; they keep no state beyond
 *    launch-configuration choices made once per process.  sg_lanczos is the
 *    one call that waits on its stream (once per restart, to read a small
 *    decision record) and writes host outputs.
 */
#ifndef SNAPGB300_H
#define SNAPGB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SG_OK 0
#define SG_ERR_ARG 1      /* invalid argument (sizes, strategy, alignment) */
#define SG_ERR_RANGE 2    /* input position outside the genome / chromosome */
#define SG_ERR_CAP 3      /* caller-provided buffer too small */
#define SG_ERR_CUDA 4     /* a CUDA launch or runtime call failed */
#define SG_ERR_NUMERIC 5  /* numerical breakdown (e.g. non-positive Gram pivot) */
#define SG_ERR_TIMEOUT 6  /* a bounded device-side wait gave up (copy never completed) */
#define SG_ERR_PARSE 7    /* malformed fragment record, or a fragment without a barcode */
#define SG_ERR_UNSORTED 8 /* sorted_by_barcode, but a barcode's records are not one run */
#define SG_ERR_CONVERT 9  /* fragment size does not fit the matrix value type (u32 / i32) */
#define SG_ERR_COLLISION 10 /* barcode hashes still collided after re-hashing (never seen) */

/* Counting strategies, same meaning as CountingStrategy in
 * snapatac2-core/src/feature_count/counter.rs:19-36 ("insertion", "fragment",
 * "paired-insertion"), plus the single-end path of gen_mat_single. */
#define SG_COUNT_INSERTION 0
#define SG_COUNT_FRAGMENT 1
#define SG_COUNT_PIC 2
#define SG_COUNT_SINGLE 3

/* Library version (major*10000 + minor*100 + patch). */
int sg_version(void);

/* Human-readable message of a status code (static storage). */
const char* sg_status_string(int status);

/* ------------------------------------------------------------------------ */
/* Tile binning: fragments -> cell x tile count matrix (CSR)                 */
/* Replaces gen_mat_pair / gen_mat_single                                    */
/*   (snapatac2-core/src/feature_count/data_iter.rs:313-415) as driven by   */
/*   create_tile_matrix (snapatac2-core/src/feature_count/matrix.rs:26-93)   */
/*   and the PyO3 entry mk_tile_matrix                                        */
/*   (snapatac2-python/src/preprocessing.rs:286-345).                        */
/*                                                                           */
/* Input is the fragment_paired encoding (import.rs:22-30): row pointer      */
/* cell_ptr[n_cells+1] (int64), frag_pos[F] = global 0-based base index of   */
/* the fragment start (uint64), frag_len[F] = fragment length (uint32).      */
/* Genome tables (device, n_chrom entries): chrom_end = cumulative base      */
/* lengths (GenomeBaseIndex base_accum_len, genome.rs:296-312), bin_off =    */
/* first output tile of each kept chromosome (0 for excluded ones),          */
/* chrom_excl = 1 if the chromosome is excluded (data_iter.rs:182-189).      */
/* min_len / max_len: fragment size bounds, -1 = none.                       */
/*                                                                           */
/* n_frags = F bounds every row pointer value (malformed rows -> SG_ERR_ARG). */
/* sg_tile_run and sg_tile_emit must get the same scratch and scratch_bytes. */
/* Three calls:                                                              */
/*  1. sg_tile_plan  -> key_ptr[n_cells+1]: exclusive prefix of the number   */
/*     of tile hits ("keys") per cell; key_ptr[n_cells] = total keys K.      */
/*  2. sg_tile_run   -> sorts and run-length-encodes each cell's keys into   */
/*     scratch (sg_tile_scratch_bytes(K) bytes) and writes out_indptr        */
/*     [n_cells+1]; out_indptr[n_cells] = nnz.                               */
/*  3. sg_tile_emit  -> copies the (tile, count) pairs into out_idx/out_cnt  */
/*     (capacity cap >= nnz).                                                */
/* The result equals the reference's CSR: per row, tile indices strictly     */
/* increasing, counts = number of hits.                                      */
/* ------------------------------------------------------------------------ */
int sg_tile_plan(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                 const uint32_t* frag_len, const uint64_t* chrom_end, const uint64_t* bin_off,
                 const uint8_t* chrom_excl, int n_chrom, uint32_t bin_size, int strategy,
                 int64_t min_len, int64_t max_len, int64_t* key_ptr, void* scan_scratch,
                 int* status, unsigned long long* bad, void* stream);

/* Bytes of scratch needed by sg_tile_plan's scan (n_cells + 1 entries). */
int64_t sg_scan_scratch_bytes(int64_t n);

/* Bytes of scratch needed by sg_tile_run for K total keys. */
int64_t sg_tile_scratch_bytes(int64_t total_keys);

int sg_tile_run(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                const uint32_t* frag_len, const uint64_t* chrom_end, const uint64_t* bin_off,
                const uint8_t* chrom_excl, int n_chrom, uint32_t bin_size, int strategy,
                int64_t min_len, int64_t max_len, const int64_t* key_ptr, void* scratch,
                int64_t scratch_bytes, int64_t* out_indptr, void* scan_scratch, int* status,
                unsigned long long* bad, void* stream);

int sg_tile_emit(int64_t n_cells, const int64_t* key_ptr, const void* scratch,
                 int64_t scratch_bytes, const int64_t* out_indptr, int32_t* out_idx,
                 uint32_t* out_cnt, int64_t cap, int* status, void* stream);


/* ------------------------------------------------------------------------ */
/* Cell-by-region counts (peak matrix) -- replaces create_peak_matrix over   */
/*   fragments (snapatac2-core/src/feature_count/matrix.rs:95-170) with     */
/*   RegionCounter::insert_fragment (feature_count/counter.rs:117-146) and   */
/*   the fragments of pair_to_fragments / single_to_fragments               */
/*   (feature_count/data_iter.rs:27-117), entered from the PyO3             */
/*   mk_peak_matrix (snapatac2-python/src/preprocessing.rs:370-430).         */
/*                                                                           */
/* Fragments as for sg_tile_plan (frag_len ignored, may be NULL, for        */
/* SG_COUNT_SINGLE).  Regions per chromosome c: [region_ptr[c],             */
/* region_ptr[c + 1]) sorted by start, chromosome coordinates, end          */
/* exclusive, region_maxend = running maximum of the ends within the        */
/* chromosome, region_id = feature index (< n_features).  A region counts   */
/* a query when start < query end and end > query start.  Strategies:      */
/* SG_COUNT_INSERTION (+1 per insertion per region), SG_COUNT_FRAGMENT      */
/* (+1 per fragment per overlapping region), SG_COUNT_PIC (+1 per region    */
/* hit by either insertion), SG_COUNT_SINGLE (single-end reads: +1 per      */
/* region containing the read's position).  min_len / max_len: size bounds  */
/* of paired fragments, -1 = none.  A position past the genome sets         */
/* SG_ERR_RANGE.  Two calls, then sg_tile_emit with the same scratch        */
/* (sg_tile_scratch_bytes(key_ptr[n_cells]) bytes): the pairs are (feature, */
/* count), features strictly increasing per row.                            */
/* ------------------------------------------------------------------------ */
int sg_region_plan(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                   const uint32_t* frag_len, const uint64_t* chrom_end, const uint8_t* chrom_excl, int n_chrom,
                   const int64_t* region_ptr, const uint64_t* region_start, const uint64_t* region_end,
                   const uint64_t* region_maxend, const uint32_t* region_id, int64_t n_features, int strategy,
                   int64_t min_len, int64_t max_len, int64_t* key_ptr, void* scan_scratch, int* status,
                   unsigned long long* bad, void* stream);
int sg_region_run(const int64_t* cell_ptr, int64_t n_cells, int64_t n_frags, const uint64_t* frag_pos,
                  const uint32_t* frag_len, const uint64_t* chrom_end, const uint8_t* chrom_excl, int n_chrom,
                  const int64_t* region_ptr, const uint64_t* region_start, const uint64_t* region_end,
                  const uint64_t* region_maxend, const uint32_t* region_id, int64_t n_features, int strategy,
                  int64_t min_len, int64_t max_len, const int64_t* key_ptr, void* scratch, int64_t scratch_bytes,
                  int64_t* out_indptr, void* scan_scratch, int* status, unsigned long long* bad, void* stream);

/* ------------------------------------------------------------------------ */
/* Fragment-file import -- replaces the PyO3 import_fragments               */
/*   (snapatac2-python/src/preprocessing.rs:87-184) and                     */
/*   snapatac2-core/src/preprocessing/import.rs:31-210 (grouping by barcode, */
/*   QC, per-cell sort) with the record syntax of qc.rs:303-348.  The file   */
/*   itself (gzip / plain) is read and decompressed by the caller; `text` is */
/*   its bytes in device memory (16-byte aligned).                           */
/*                                                                           */
/*   1. sg_frag_count_lines  -> number of lines (synchronises the stream)    */
/*   2. sg_frag_index_lines  -> line_start[n_lines + 1]                      */
/*   3. sg_frag_import       -> everything in `workspace`; sizes in info     */
/*   4. sg_frag_emit         -> copies the results into exact-size arrays    */
/* ------------------------------------------------------------------------ */

/* Bytes of scratch for sg_frag_count_lines / sg_frag_index_lines.          */
int64_t sg_frag_line_scratch_bytes(int64_t nbytes);
/* *n_lines (host) = number of '\n' plus one for an unterminated last line. */
int sg_frag_count_lines(const uint8_t* text, int64_t nbytes, void* scratch, int64_t* n_lines, void* stream);
/* line_start[i] = first byte of line i; line_start[n_lines] = nbytes, or   */
/* nbytes + 1 when the last line has no newline.  Same scratch as above.    */
int sg_frag_index_lines(const uint8_t* text, int64_t nbytes, const void* scratch, int64_t n_lines,
                        int64_t* line_start, void* stream);

/* Bytes of workspace for sg_frag_import / sg_frag_emit (about 300 B per    */
/* line plus 32 B per whitelist entry).                                      */
int64_t sg_frag_workspace_bytes(int64_t n_lines, int64_t n_whitelist);

/* The import (import_fragments, snapatac2-core/src/preprocessing/          */
/* import.rs:31-210, entered from preprocessing.rs:87-184 of the Python     */
/* package).  Chromosomes: n_chrom names sorted by bytes (chrom_blob +      */
/* chrom_off[n_chrom + 1]), their lengths, the cumulative length before each */
/* (chrom_base) and a mitochondrial flag per name; genome_size = total.      */
/* Whitelist (has_whitelist != 0): n_whitelist byte strings (wl_blob +       */
/* wl_off[n_whitelist + 1]).  min_num_fragments, sorted_by_barcode,          */
/* shift_left, shift_right as in the reference; seed: barcode hash seed.     */
/* info (host, 10 entries): [0] cells, [1] matrix entries, [2] paired (1),   */
/* single-end (0) or no record (-1), [3] line of the first error or -1,      */
/* [4] records with a barcode, [5] distinct barcodes, [6] re-hashes,         */
/* [7] matrix sort path (0 = one 64-bit key, 1 = three keys), [8] kernels    */
/* launched, [9] reserved.  Synchronous:                                     */
/* returns after the stream has finished.  Errors: SG_ERR_PARSE (malformed   */
/* line, or a fragment without a barcode), SG_ERR_UNSORTED, SG_ERR_RANGE     */
/* (position past its chromosome), SG_ERR_CONVERT; info[3] names the line.   */
int sg_frag_import(const uint8_t* text, int64_t nbytes, const int64_t* line_start, int64_t n_lines,
                   const uint8_t* chrom_blob, const int64_t* chrom_off, const uint64_t* chrom_size,
                   const uint64_t* chrom_base, const uint8_t* chrom_mito, int n_chrom, uint64_t genome_size,
                   const uint8_t* wl_blob, const int64_t* wl_off, int64_t n_whitelist, int has_whitelist,
                   uint64_t min_num_fragments, int sorted_by_barcode, int64_t shift_left, int64_t shift_right,
                   uint64_t seed, void* workspace, int64_t workspace_bytes, int64_t* info, void* stream);

/* Results of sg_frag_import (same n_lines, n_whitelist and info):         */
/* out_indptr[cells + 1], out_indices[entries] (global base index),         */
/* out_data[entries] (uint32 size for paired data, int32 signed size for    */
/* single-end data), and per cell: barcode location in `text` (byte offset  */
/* << 16 | length), n_fragment, frac_dup, frac_mito (qc.rs:454-465).        */
int sg_frag_emit(const void* workspace, int64_t n_lines, int64_t n_whitelist, const int64_t* info,
                 int64_t* out_indptr, int64_t* out_indices, int32_t* out_data, uint64_t* out_bc_loc,
                 uint64_t* out_n_fragment, double* out_frac_dup, double* out_frac_mito, void* stream);

/* Stable LSD radix sort of n uint64 keys (and uint64 payloads when vals is */
/* not NULL) by key bits [begin_bit, end_bit), 8 bits per pass, between the */
/* buffers (keys, vals) and (keys_alt, vals_alt); *result_in_alt (host) = 1 */
/* when the result ended in the _alt buffers.  Used by the import; exported */
/* for tests.  No reference counterpart (the reference sorts on the host).  */
int64_t sg_radix_scratch_bytes(int64_t n);
int sg_radix_sort_u64(int64_t n, uint64_t* keys, uint64_t* vals, uint64_t* keys_alt, uint64_t* vals_alt,
                      int begin_bit, int end_bit, void* scratch, int* result_in_alt, void* stream);

/* ------------------------------------------------------------------------ */
/* Row and segment steps around the main kernels                            */
/* ------------------------------------------------------------------------ */

/* Rows `rows[k]` of a CSR, in that order (the Nyström landmark matrix,     */
/* `slice(&[selected_samples, ...])`, snapatac2-python/src/embedding.rs:95-99). */
/* sg_csr_row_ptr writes out_ptr[k + 1] (scan_scratch: sg_scan_scratch_bytes(k)); */
/* sg_csr_copy_rows then copies indices (and values when not NULL).        */
int sg_csr_row_ptr(int64_t k, const int64_t* rows, const int64_t* indptr, int64_t* out_ptr, void* scan_scratch,
                   void* stream);
int sg_csr_copy_rows(int64_t k, const int64_t* rows, const int64_t* indptr, const int32_t* indices,
                     const float* values, const int64_t* out_ptr, int32_t* out_idx, float* out_val, void* stream);

/* dst[dst_off[i] ..] = src[off[i] .. off[i] + len[i]) for i < k: the cell  */
/* barcodes of an import gathered out of the fragment text.                 */
int sg_gather_bytes(int64_t k, const int64_t* off, const int32_t* len, const int64_t* dst_off, const uint8_t* src,
                    uint8_t* dst, void* stream);

/* Gene-level counts: per row, the maximum count over the regions mapped to */
/* each gene (GeneCount::get_values, snapatac2-core/src/feature_count/      */
/* counter.rs:270-283).  Input: a region-count CSR (n rows, nnz entries,    */
/* region indices, uint32 counts) and region_gene[region].  Output: out_ptr */
/* [n + 1], out_idx / out_val (room for nnz entries; genes ascending within */
/* a row), *n_out (host) = entries written.  Synchronises the stream.       */
int64_t sg_gene_max_scratch_bytes(int64_t nnz);
int sg_gene_max(int64_t n, const int64_t* indptr, const int32_t* region, const uint32_t* counts,
                const int32_t* region_gene, int64_t nnz, void* scratch, int64_t scratch_bytes, int64_t* out_ptr,
                int32_t* out_idx, int32_t* out_val, int64_t* n_out, void* stream);

/* Nyström's per-chunk rescaling (the embedded Python of `nystrom`,         */
/* snapatac2-python/src/embedding.rs:222-229) of q[n][k] (FP64, k <= 256) in */
/* place, chunks of `chunk` rows: t = λ ⊙ Σ_chunk q, d = q t, d <= 0 -> the  */
/* chunk's smallest positive d, q /= sqrt(d).  A chunk with no positive d   */
/* where one is needed sets status SG_ERR_NUMERIC, bad = its first row.     */
int sg_nystrom_rescale(int64_t n, int k, double* q, const double* evals, int64_t chunk, int* status,
                       unsigned long long* bad, void* stream);

/* ------------------------------------------------------------------------ */
/* Feature selection -- the `count` vector of select_features              */
/*   (snapatac2-python/python/snapatac2/preprocessing/_basic.py:1053-1056:   */
/*   FP64 column sums of X).  The ranking itself (_basic.py:952-967, NumPy  */
/*   argsort tie order) stays with the caller.                               */
/* ------------------------------------------------------------------------ */

/* out[m] = column sums of the CSR entries.  counts (uint32) or values      */
/* (float32) or neither (binary pattern: 1 per entry), not both.  Integer   */
/* inputs are summed exactly in uint64 (scratch: m uint64) and converted:    */
/* identical to the reference's FP64 sums.  Float values are summed in FP64  */
/* (scratch unused).  Out-of-range column indices set status SG_ERR_ARG      */
/* with the first offending entry in bad.                                    */
int sg_col_counts(int64_t nnz, int64_t m, const int32_t* indices, const uint32_t* counts, const float* values,
                  double* out, unsigned long long* scratch, int* status, unsigned long long* bad, void* stream);

/* ------------------------------------------------------------------------ */
/* Spectral embedding (matrix-free cosine) -- replaces spectral_embedding    */
/*   (snapatac2-python/src/embedding.rs:24-59): column slice + idf +         */
/*   normalize + spectral_mf degree (embedding.rs:133-152,269-286,315-326)   */
/*   and the SciPy ARPACK eigsh call on X̂X̂ᵀ - D⁻¹ (embedding.rs:155-188).    */
/*                                                                           */
/* Matrices are CSR with int64 row pointers and int32 column indices, rows   */
/* sorted and unique.  values == NULL means the implicit 1.0 pattern.        */
/* dtype: 0 = float32 (mixed precision), 1 = float64.                        */
/* ------------------------------------------------------------------------ */

/* Keep the entries whose column maps to colmap[col] >= 0, renumbered to     */
/* colmap[col] (X[:, selected_features], embedding.rs:36-41).  out_indices /  */
/* out_values need capacity nnz(input); out_indptr[n] = kept nnz.  Column    */
/* indices are not checked: each must index colmap (caller's check).        */
int sg_csr_select_cols(int64_t n, const int64_t* indptr, const int32_t* indices, const float* values,
                       const int32_t* colmap, int64_t* out_indptr, int32_t* out_indices, float* out_values,
                       void* scan_scratch, void* stream);

/* Number of row blocks used by sg_csr_transpose.                          */
int sg_transpose_blocks(void);

/* Bytes of scratch (256-B aligned) sg_csr_transpose needs.                 */
int64_t sg_transpose_work_bytes(int64_t n, int64_t m, int nblk);

/* Deterministic CSR -> CSC transpose (rows ascending in every column).     */
/* colptr[m+1] (int64), rowidx[nnz], cvalues[nnz] (NULL if values NULL).     */
/* Unsorted / duplicate / out-of-range column indices -> status SG_ERR_ARG   */
/* (the outputs are then not written).                                       */
int sg_csr_transpose(int64_t n, int64_t m, const int64_t* indptr, const int32_t* indices,
                     const float* values, int nblk, void* work, int64_t work_bytes, int64_t* colptr,
                     int32_t* rowidx, float* cvalues, void* scan_scratch, int* status, void* stream);

/* Operator set-up in FP64: w = idf (or a copy of feature_weights when not  */
/* NULL), w2 = w², rinv = 1/||(XW)_i||, colsum = 1ᵀXn, dinv = 1/(d - 1),    */
/* a = rinv * sqrt(dinv); float copies w2_32/a32/dinv32 may be NULL.        */
/* minmax: 2 uint64 of scratch.  A zero row or a non-positive d - 1 sets    */
/* status SG_ERR_NUMERIC with the row in bad (the reference yields NaN).     */
int sg_spectral_prepare(int64_t n, int64_t m, const int64_t* indptr, const int32_t* indices,
                        const float* values, const int64_t* colptr, const int32_t* rowidx,
                        const float* cvalues, const double* feature_weights, double* w, double* w2,
                        float* w2_32, double* rinv, double* colsum, double* a, double* dinv, float* a32,
                        float* dinv32, unsigned long long* minmax, int* status, unsigned long long* bad,
                        void* stream);

/* SpMM over a block of `block` (4, 8, 16, 32) dense columns:               */
/*   out[r,:] = scale[r] * sum_{e in row r} val_e * in[col_e,:]              */
/*              - dshift[r] * y[r,:]            (when dshift != NULL)       */
/* in/out/y row-major with row stride = block.  grid <= 0: default grid.    */
/* The Gram matvec is two calls: T = w2 ⊙ Xᵀ(a ⊙ V) over the CSC, then     */
/* W = a ⊙ X T - dinv ⊙ V over the CSR.                                      */
int sg_spmm(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
            const void* in, void* out, const void* scale, const void* dshift, const void* y, int grid,
            void* stream);

/* sg_spmm with an explicit memory-access variant in [0, sg_spmm_variants()) */
/* (same arithmetic and result; an autotuner picks the fastest per shape).   */
int sg_spmm_variants(void);
int sg_spmm_ex(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
               const void* in, void* out, const void* scale, const void* dshift, const void* y, int grid,
               int variant, void* stream);

/* sg_spmm_ex that skips (does not write) the rows with row_mask[r] == 0.    */
int sg_spmm_masked(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
                   const void* in, void* out, const void* scale, const void* dshift, const void* y, int grid,
                   int variant, const unsigned char* row_mask, void* stream);

/* IDF weights from per-column cell counts (FP64, e.g. sg_col_counts of the */
/* index pattern) with the rules of idf (embedding.rs:269-286): all counts   */
/* equal -> 1, count 0 -> 1, count n -> n - 1, w = ln(n / count).  mm: two   */
/* uint64 of scratch.                                                       */
int sg_idf_from_counts(int64_t n, int64_t m, const double* counts, double* w, unsigned long long* mm,
                       void* stream);

/* rinv[i] = 1 / ||x_i ⊙ w||_2 over the CSR rows (normalize, embedding.rs:  */
/* 315-326); a row with no weight sets SG_ERR_NUMERIC with its index.        */
/* Column indices are not checked: each must index w (caller's check).       */
int sg_csr_row_norms(int64_t n, const int64_t* indptr, const int32_t* indices, const float* values,
                     const double* w, double* rinv, int* status, unsigned long long* bad, void* stream);

/* sg_spmm_masked on a persistent grid whose warps take 4 rows at a time    */
/* from *counter (device, zeroed by this call on `stream`): rows of very     */
/* different lengths leave no tail.  Same per-row arithmetic and result.     */
/* FP32 only (dtype 0); variant as for sg_spmm_ex; rows < 2^31.  Calls that  */
/* run concurrently need separate counters.  No reference counterpart (a    */
/* schedule of the Gram matvec of embedding.rs:155-188).                    */
int sg_spmm_dyn(int dtype, int block, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val,
                const void* in, void* out, const void* scale, const void* dshift, const void* y, int variant,
                const unsigned char* row_mask, unsigned int* counter, void* stream);
/* sg_spmm_dyn over a row order: the counter walks `positions` positions and */
/* order[p] (device int32, -1 = none) is the row at position p.  With the   */
/* order of sg_row_order the longest rows are taken first, one per 4-row     */
/* fetch, so the last rows to finish are short (longest-first scheduling of */
/* the Xᵀ pass, whose rows are features of very different lengths).  Same   */
/* per-row arithmetic and result as sg_spmm_dyn.  No reference counterpart. */
int sg_spmm_dyn_ordered(int dtype, int block, int64_t positions, const int64_t* ptr, const int32_t* idx,
                        const float* val, const void* in, void* out, const void* scale, const void* dshift,
                        const void* y, int variant, const int32_t* order, unsigned int* counter, void* stream);
/* Row order of a CSR by descending row length (ties: ascending row), dealt */
/* so that position 4c + j holds the row of rank c + j * ceil(rows / 4):    */
/* order has sg_row_order_positions(rows) entries; scratch of               */
/* sg_row_order_scratch_bytes(rows) bytes, 256-byte aligned.                */
int64_t sg_row_order_positions(int64_t rows);
int64_t sg_row_order_scratch_bytes(int64_t rows);
int sg_row_order(int64_t rows, const int64_t* ptr, int32_t* order, void* scratch, int64_t scratch_bytes, void* stream);

/* Stage-tiled SpMM, same result contract as sg_spmm_masked (summation     */
/* order differs at rounding level).  One CTA per SM (and wave) owns a row  */
/* range; the dense operand `in` (cols x block, every row is read) streams  */
/* through shared memory in column stages by bulk asynchronous copies,      */
/* together with each stage's segment table (per row: the [start, end) of   */
/* its nonzeros in the stage), built once by sg_staged_table for the matrix */
/* and the (dtype, block) row width.  in/out/y/table 16-byte aligned; out   */
/* must not alias in.  A stage copy that never completes sets               */
/* *status = SG_ERR_TIMEOUT (bounded 2 s wait).  Variants in                */
/* [0, sg_spmm_staged_variants()) differ in lanes per row and unroll.        */
int sg_spmm_staged_variants(void);
/* Bytes of the segment table for this shape (0: shape not supported).      */
int64_t sg_staged_table_bytes(int dtype, int block, int64_t rows, int64_t cols);
int sg_staged_table(int dtype, int block, int64_t rows, int64_t cols, const int64_t* ptr, const int32_t* idx,
                    void* table, int64_t table_bytes, void* stream);
int sg_spmm_staged(int dtype, int block, int64_t rows, int64_t cols, const int64_t* ptr, const int32_t* idx,
                   const float* val, const void* table, const void* in, void* out, const void* scale,
                   const void* dshift, const void* y, int variant, const unsigned char* row_mask, int* status,
                   void* stream);

/* Compensated-FP32 SpMM over 32 columns, used by the FP64 correction sweep */
/* of sg_lanczos (the Gram matvec of embedding.rs:133-152 applied once to   */
/* the Ritz vectors).  Operands are FP32 pairs (hi, lo) whose sum is the    */
/* FP64 value (sg_ds_split); sums are carried as an FP32 value and an FP32  */
/* compensation updated by Knuth's TwoSum, within about k * 2^-48 of the    */
/* sum of |terms| for k terms.  `in` is rows' cols x 32 pairs (256 B a row). */
/* pass 0: out = pairs of scale ⊙ (M in)              (dshift must be NULL) */
/* pass 1: out = scale ⊙ (M in) - dshift ⊙ y, FP64 x 32 (y FP64, rows x 32)  */
/* M is the CSR (ptr, idx, val; val NULL: all ones).  in, out, y 16-byte    */
/* aligned; out must not alias in.  Variants 0-3: one or two 32-index       */
/* chunks in flight (bit 0), static or counter-driven row schedule (bit 1,  */
/* needs `counter`, zeroed by the call).  `order` (counter-driven variants  */
/* only, else NULL): a row order as for sg_spmm_dyn_ordered, `rows` then    */
/* being its number of positions.  Deterministic.  No reference             */
/* counterpart (an arithmetic form of the FP64 matvec).                     */
int sg_spmm_ds_variants(void);
int sg_spmm_ds(int pass, int64_t rows, const int64_t* ptr, const int32_t* idx, const float* val, const void* in,
               void* out, const double* scale, const double* dshift, const double* y, int variant,
               const int32_t* order, unsigned int* counter, void* stream);
/* out[r, c] = (hi, lo) pair of a[r] * U[r, c] (a NULL: of U[r, c]); U is   */
/* n x 32 FP64, out n x 32 pairs of FP32 (hi = fl32(v), lo = fl32(v - hi)). */
int sg_ds_split(int64_t n, const double* a, const double* U, void* out, void* stream);

/* Diagnostic (no reference counterpart): the row gathers of one SpMM pass  */
/* alone -- table[idx[e]] (block values per row, same 16-byte vectors and    */
/* lanes per row as the SpMM) for every e < nnz, folded into registers, no   */
/* output.  Its time over a matrix's index stream is the floor the SpMM      */
/* pass can reach with this access pattern.  sink: one float, written only   */
/* in a case that does not occur for finite tables.                          */
int sg_gather_ceiling(int dtype, int block, int64_t nnz, const int32_t* idx, const void* table, float* sink,
                      void* stream);

/* ---- block Krylov-Schur (thick-restart block Lanczos) building blocks --- */
/* Together they replace the ARPACK eigsh call of eigen                      */
/* (snapatac2-python/src/embedding.rs:155-188; ARPACK itself is SciPy's).    */
/* Q: n x ldq row-major basis; W: n x block working block.                   */

/* Number of per-CTA partials of the projections (part = parts*ncols*block). */
int sg_proj_parts(void);

/* count values uniform in [-0.5, 0.5) from a hash of (seed, index): the    */
/* start block of the eigensolver, identical on every platform.             */
int sg_fill_random(int dtype, int64_t count, uint64_t seed, void* out, void* stream);

/* C (ncols x block, FP64) = Q[:, :ncols]ᵀ W.                               */
int sg_block_proj(int dtype, int block, int64_t n, const void* Q, int64_t ldq, int ncols, const void* W,
                  double* part, int nparts, double* C, void* stream);

/* W -= Q[:, :ncols] C.                                                      */
int sg_block_update(int dtype, int block, int64_t n, const void* Q, int64_t ldq, int ncols, const double* C,
                    void* W, void* stream);

/* One Cholesky-QR pass: G = WᵀW = RᵀR, W <- W R⁻¹ (G, R, Rinv FP64).        */
/* A rank-deficient block sets status SG_ERR_NUMERIC.                        */
int sg_block_cholqr(int dtype, int block, int64_t n, void* W, double* part, int nparts, double* G, double* R,
                    double* Rinv, int* status, void* stream);

/* Q[:, col:col+block] = W; Z = W; Zs = rowscale ⊙ W (NULL pointers skip).   */
int sg_block_finish(int dtype, int block, int64_t n, const void* W, void* Q, int64_t ldq, int col, void* Z,
                    void* Zs, const void* rowscale, void* stream);

/* H[m0:m0+b, m0:m0+b] = sym(C1 + C2)[m0:m0+b]; Rout = R2 R1; if            */
/* write_coupling, H[m0+b:m0+2b, m0:m0+b] = Rout and its transpose.          */
int sg_lanczos_hblock(int block, double* H, int64_t ldh, int m0, const double* C1, const double* C2,
                      const double* R1, const double* R2, double* Rout, int write_coupling, void* stream);

/* out[:, 0:k] = Q[:, 0:m] Y[0:m, 0:k] (tq/to: 0 = float, 1 = double).       */
int sg_basis_rotate(int tq, int to, int64_t n, const void* Q, int64_t ldq, int m, const double* Y,
                    int64_t ldy, int k, void* out, int64_t ldo, void* stream);

/* Eigenpairs of a symmetric n x n FP64 matrix on the GPU (n <= 640): the q  */
/* smallest and p largest eigenvalues (all n when p + q >= n), ascending,    */
/* into evals (device), their unit eigenvectors as the rows of evecs         */
/* (device, count x n), largest component positive.  Householder reduction   */
/* on one thread-block cluster, multisection and inverse iteration.  This is */
/* the Rayleigh-Ritz step of sg_lanczos, exported for tests and callers.     */
/* Replaces the small dense eigensolve inside ARPACK (embedding.rs:155-171). */
int64_t sg_sym_eig_work_bytes(int n, int p, int q);
int sg_sym_eig(int n, const double* A, int64_t lda, int p, int q, double* evals, double* evecs, void* work,
               int64_t work_bytes, void* stream);

/* ---- one-call eigensolver: replaces eigen (embedding.rs:155-188) ------- */
/* The operator A v = a ⊙ (X (w² ⊙ (Xᵀ (a ⊙ v)))) - dinv ⊙ v of one dataset, */
/* as sg_csr_transpose and sg_spectral_prepare leave it; the reference       */
/* builds the same operator in spectral_mf (embedding.rs:133-152) and hands  */
/* it to eigsh.  All pointers are device pointers.                           */
typedef struct sg_gram_op {
  int64_t n, m;                                 /* cells, features            */
  const int64_t* indptr;                        /* X, CSR (n + 1)             */
  const int32_t* indices;                       /*                            */
  const float* values;                          /* NULL: binary pattern       */
  const int64_t* colptr;                        /* X, CSC (m + 1)             */
  const int32_t* rowidx;                        /*                            */
  const float* cvalues;                         /* NULL: binary pattern       */
  const double* w2;                             /* FP64 scalings (m, n, n)    */
  const double* a;
  const double* dinv;
  const float* w2_f32;                          /* FP32 copies (mixed form)   */
  const float* a_f32;
  const float* dinv_f32;
  const void* staged_table_t;                   /* stage-tiled SpMM segment   */
  const void* staged_table_x;                   /* tables, or NULL            */
  const int32_t* order_t;                       /* sg_row_order of the CSC    */
  int64_t order_t_positions;                    /* (longest columns first for */
                                                /* the dynamic Xᵀ pass), or   */
                                                /* NULL / 0                   */
} sg_gram_op;

/* Solver settings; zero / negative fields take the defaults (a NULL opts   */
/* pointer: all defaults, the correction sweep on, default SpMM kernels).   */
typedef struct sg_lanczos_opts {
  int basis;                /* Krylov basis size M (multiple of block)       */
  int keep;                 /* thick-restart size                            */
  double tol_vec;           /* residual bar (x max|θ|) of returned vectors,  */
                            /* default 3e-9                                  */
  double tol_val;           /* residual bar of the other wanted pairs        */
  int vec_positive_only;    /* 1: vectors returned for θ > 0 only (as        */
                            /* weighted_by_sd keeps), others need tol_val    */
  int max_restarts;         /* < 0: default 200 (0: no restart)              */
  int refine;               /* mixed form: final correction sweep (FP64-    */
                            /* class AU, Rayleigh-Ritz in FP64): 1 with the  */
                            /* compensated FP32 kernels (sg_spmm_ds), 2 with */
                            /* FP64 kernels, 0 none                          */
  int variant_t, variant_x; /* SpMM kernel per pass (codes: < 100 gather,    */
                            /* 100 + v stage-tiled, 200 + v dynamic); -1:    */
                            /* library default                               */
  int refine_variant_t, refine_variant_x; /* SpMM of the sweep: refine 1,  */
                            /* sg_spmm_ds variants 0-3; refine 2, FP64      */
                            /* block-32 gather or dynamic codes; -1 default  */
  int time_spmm;            /* 1: CUDA-event time of every SpMM launch       */
} sg_lanczos_opts;

typedef struct sg_lanczos_info {
  int64_t block_matvecs;
  int32_t restarts;
  int32_t converged;        /* every wanted pair met its bar                 */
  int32_t basis, keep;
  double max_residual;      /* largest Ritz residual of the returned pairs   */
  double next_evals[4];     /* Ritz values just outside the wanted set       */
  double seconds_cycles;    /* host wall time of the expansion cycles,       */
  double seconds_ritz;      /* of the GPU Rayleigh-Ritz steps (incl. the     */
  double seconds_restart;   /* read of their decision), of the restarts and  */
  double seconds_refine;    /* of the final rotation and correction sweep    */
  double spmm_ms_t, spmm_ms_x; /* CUDA-event time of the SpMM passes         */
  int64_t spmm_launches;
  int64_t kernel_launches;  /* kernels this call launched                    */
} sg_lanczos_info;

int64_t sg_lanczos_work_bytes(int precision, int block, int k, int64_t n, int64_t m, int basis, int keep);

/* The k eigenpairs of largest magnitude (eigsh which='LM'), eigenvalues     */
/* descending into evals (host, k), eigenvectors into evecs (device, n x k   */
/* FP64 row-major), Ritz residual estimates into residuals (host, k; NULL    */
/* skips).  precision 0: FP32 SpMM and basis, FP64 Rayleigh-Ritz (mixed);    */
/* 1: all FP64.  block: 4, 8, 16 or 32.  Thick-restart block Lanczos with    */
/* full reorthogonalisation; the restart's Rayleigh-Ritz runs on the GPU in  */
/* FP64 (sg_sym_eig) and the host reads one small decision record per        */
/* restart.  work: caller-owned, 256-byte aligned, sg_lanczos_work_bytes.    */
/* status: device int (zeroed here).  Returns SG_ERR_NUMERIC for a rank-     */
/* deficient Krylov block; an unconverged solve is not an error            */
/* (info->converged = 0).  Host arguments (evals, residuals, info) are       */
/* written before it returns; evecs is complete when the stream is.         */
int sg_lanczos(const sg_gram_op* op, int precision, int block, int k, uint64_t seed, const sg_lanczos_opts* opts,
               void* work, int64_t work_bytes, double* evals, double* evecs, double* residuals,
               sg_lanczos_info* info, int* status, void* stream);

/* ------------------------------------------------------------------------ */
/* Aggregation of an existing cell x feature matrix by regions (use_x=True  */
/* of the peak and gene matrices) -- replaces read_chrom_values().           */
/*   aggregate_by(counter) in create_peak_matrix / create_gene_matrix        */
/*   (snapatac2-core/src/feature_count/matrix.rs:121-128,211-218,           */
/*   data_iter.rs:866-891): each entry (feature j, value v) adds v to every  */
/*   region overlapping feature j's interval (RegionCounter::insert,         */
/*   counter.rs:95-106).  fptr/fregion: CSR of the feature -> region map     */
/*   (region ids < n_regions).  Two calls: sg_csr_aggregate_count writes     */
/*   eoff[n+1] (exclusive offsets of each row's expanded records, total at   */
/*   eoff[n]); sg_csr_aggregate_run (scratch of                              */
/*   sg_csr_aggregate_scratch_bytes(n, total) bytes, 256-byte aligned)       */
/*   writes out_indptr[n+1], out_idx (regions ascending per row), out_val    */
/*   (dtype 0: uint32 sums, status SG_ERR_CONVERT past 2^32-1; 1: FP64 sums  */
/*   in X's column order) and the entry count to the host *out_nnz; it       */
/*   synchronises its stream once; SG_ERR_CAP if cap < nnz (*out_nnz set).   */
/* ------------------------------------------------------------------------ */
int sg_csr_aggregate_count(int64_t n, const int64_t* indptr, const int32_t* indices, const int64_t* fptr,
                           int64_t* eoff, void* scan_scratch, void* stream);
int64_t sg_csr_aggregate_scratch_bytes(int64_t n, int64_t n_records);
int sg_csr_aggregate_run(int dtype, int64_t n, const int64_t* indptr, const int32_t* indices, const void* values,
                         const int64_t* fptr, const int32_t* fregion, int64_t n_regions, const int64_t* eoff,
                         int64_t n_records, void* scratch, int64_t scratch_bytes, int64_t* out_indptr,
                         int32_t* out_idx, void* out_val, int64_t cap, int64_t* out_nnz, int* status, void* stream);

/* ------------------------------------------------------------------------ */
/* Exact kNN graph -- replaces nearest_neighbour_graph                       */
/*   (snapatac2-python/src/knn.rs:7-16 -> snapatac2-core/src/utils/knn.rs:  */
/*   9-31, to_csr_matrix 58-78).                                             */
/* X: n x d row-major FP64 (d <= 64).  Output: nbr (n x k int64) and dist    */
/* (n x k FP64 = sqrt of the squared Euclidean distance), each row sorted by */
/* neighbour index, self excluded by index; identical to the FP64 kNN except */
/* for the order of exact distance ties (smaller index first).               */
/* margin: extra FP32 candidates per query (k + margin <= 128 is used).       */
/* *n_fallback (device int, may be NULL) = number of queries that needed the */
/* exact FP64 rescan.  scratch: sg_knn_scratch_bytes bytes, 256-B aligned.   */
/* ------------------------------------------------------------------------ */
int64_t sg_knn_scratch_bytes(int64_t n, int d, int k, int margin);

int sg_knn(const double* X, int64_t n, int d, int k, int margin, int64_t* nbr, double* dist, void* scratch,
           int64_t scratch_bytes, int* n_fallback, void* stream);

/* ------------------------------------------------------------------------ */
/* Batched Krylov-Schur over many datasets stacked block-diagonally (rows   */
/* roff[d]..roff[d+1] belong to dataset d).  CTA partition of the rows:     */
/* cta_r0/cta_r1 (never crossing a dataset), CTAs of dataset d are          */
/* ds_cta[d]..ds_cta[d+1].  active[d] == 0 freezes dataset d.  C/G/R/H hold */
/* one block per dataset (strides as documented per call).  No counterpart  */
/* in the reference, which embeds one dataset per call.                     */
/* ------------------------------------------------------------------------ */
int sg_bblock_proj(int dtype, int block, int D, int ncta, const int* ds_cta, const int* cta_ds, const int* active,
                   const int64_t* cta_r0, const int64_t* cta_r1, const void* Q, int64_t ldq, int ncols,
                   const void* W, double* part, double* C, int64_t cstride, void* stream);
int sg_bblock_update(int dtype, int block, int64_t nrows, int D, const int64_t* roff, const int* active,
                     const void* Q, int64_t ldq, int ncols, const double* C, int64_t cstride, void* W, void* stream);
int sg_bblock_cholqr(int dtype, int block, int64_t nrows, int D, const int64_t* roff, const int* active, int ncta,
                     const int* ds_cta, const int* cta_ds, const int64_t* cta_r0, const int64_t* cta_r1, void* W,
                     double* part, double* G, double* R, double* Rinv, int* status, int* bad_ds, void* stream);
/* mask[i] = active[d] for the dataset d holding index i (offsets off[D+1]); */
/* the row masks of sg_spmm_masked for frozen datasets.                      */
int sg_bmask(int64_t n, int D, const int64_t* off, const int* active, unsigned char* mask, void* stream);
int sg_blanczos_hblock(int block, int D, const int* active, double* H, int64_t ldh, int m0, const double* C1,
                       const double* C2, int64_t cstride, const double* R1, const double* R2, double* Rout,
                       void* stream);
int sg_bbasis_rotate(int tq, int to, int ncta, const int* cta_ds, const int64_t* cta_r0, const int64_t* cta_r1,
                     const void* Q, int64_t ldq, int m, const double* Y, int64_t ldy, int64_t ystride, int k,
                     void* out, int64_t ldo, void* stream);
/* Per-dataset IDF on stacked columns (coff column offsets), the rules of   */
/* idf (snapatac2-python/src/embedding.rs:269-286) with n = the dataset's   */
/* cell count.  minmax: 2*D uint64 scratch.                                 */
int sg_bidf(int64_t m, const int64_t* colptr, int D, const int64_t* coff, const int64_t* roff,
            unsigned long long* minmax, double* w, void* stream);

/* ------------------------------------------------------------------------ */
/* Adjoint: gradient of the sum of the wanted eigenvalues of the cosine     */
/* operator with respect to the feature weights (no counterpart in the      */
/* reference, whose weights are fixed inputs, embedding.rs:42-47).  FP64.   */
/* U: n x k eigenvectors (row-major), evals: k, dinv/rinv from              */
/* sg_spectral_prepare.  Between the stages the caller runs sg_spmm in FP64:*/
/*   stage1 -> [r s U | r δ̄ | r] (n x block)   ; CSC SpMM -> ZEH (m x block) */
/*   stage2 -> [w² Z | w² e]     (m x block2)  ; CSR SpMM -> P   (n x block2)*/
/*   stage3 -> [ρ̄ r, 0, 0, 0]    (n x 4)       ; CSC SpMM with squared      */
/*                                              values -> g (m x 4)          */
/*   final  -> grad[m]                                                       */
/* ------------------------------------------------------------------------ */
int sg_adjoint_stage1(int64_t n, int k, const double* U, const double* evals, const double* dinv,
                      const double* rinv, int block, double* out, double* dbar, void* stream);
int sg_adjoint_stage2(int64_t m, int k, const double* zeh, int block, const double* w, int block2, double* out,
                      void* stream);
int sg_adjoint_stage3(int64_t n, int k, const double* U, const double* dinv, const double* rinv,
                      const double* dbar, const double* P, int block2, double* out, void* stream);
int sg_adjoint_final(int64_t m, int k, const double* w, const double* zeh, int block, const double* g,
                     double* grad, void* stream);
/* out[t] = values[t]^2 (the X∘X values of the third SpMM). */
int sg_square_values(int64_t nnz, const float* values, float* out, void* stream);

/* Test hook (no counterpart in the reference): the stage-tiled SpMM skips  */
/* the copies of stage skip_stage, so that stage's bounded wait runs out    */
/* with nothing in flight (status SG_ERR_TIMEOUT, the kernel returns), and  */
/* every stage wait gives up after wait_ns.  skip_stage < 0, wait_ns <= 0:  */
/* normal operation.  Synchronous; process-wide; for failure tests only.    */
int sg_test_staged_fault(int skip_stage, int64_t wait_ns);

/* Allocation-free sg_knn (no counterpart in the reference).  Same inputs,   */
/* outputs and result as sg_knn, for callers that cannot allocate device    */
/* memory: the scratch is a fixed array inside the library (about 33 MB per  */
/* GPU that loads it, held until exit).  Limits: n <= 16384 points,          */
/* d <= 32, k <= 100 (k + margin is capped at 128); larger problems return   */
/* SG_ERR_CAP without touching the outputs.  Every call looks up the array's */
/* device address (cudaGetSymbolAddress, with the caller's device current),  */
/* so the address stays right after cudaDeviceReset; the first call on a    */
/* device also loads the library's device code there (lazy module loading),  */
/* so make that first call before any stream capture.                        */
/* All calls share the one array: calls that overlap on the GPU (different   */
/* streams, no ordering between them) race and must be avoided.             */
int sg_knn_noalloc(const double* X, int64_t n, int d, int k, int margin, int64_t* nbr, double* dist,
                   int* n_fallback, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* SNAPGB300_H */
