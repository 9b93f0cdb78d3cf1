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
 *  - Entry points are re-entrant per stream; they keep no state.
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

#ifdef __cplusplus
}
#endif

#endif /* SNAPGB300_H */
