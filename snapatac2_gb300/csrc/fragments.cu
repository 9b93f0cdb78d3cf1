// Fragment-file import (snap.pp.import_fragments) on the GPU.
//
// Input: the decompressed text of a fragment file in device memory.  Output:
// the per-cell fragment matrix of the reference (rows = cells, column = global
// base index of the fragment start, value = fragment size; signed size for
// single-end reads) plus the per-cell QC columns.  Reference:
// snapatac2-python/src/preprocessing.rs:87-184 (entry, shifts, unsorted
// input) and snapatac2-core/src/preprocessing/import.rs:31-210 (grouping,
// QC, per-cell sort), record syntax qc.rs:303-348.
//
// Pipeline (one CUDA stream; the host reads back a handful of sizes):
//   lines     newline count per 64 KB chunk, scan, line starts;
//   parse     thread per line: fields, saturating shifts, chromosome by
//             binary search over the sorted names, global position and
//             signed size, 64-bit barcode hash (SplitMix64 finaliser over
//             8-byte words), flags;
//   group     records with a barcode compacted and radix-sorted by hash;
//             equal hashes are checked byte for byte (a collision re-hashes
//             with another seed), group ids by scan, per-group counts by
//             warp-segmented reductions and one atomic per run;
//   decide    whitelist (hash + byte compare), the minimum-count whitelist
//             of unsorted input, the "sorted by barcode" check (a group's
//             records must be one run), position and size-conversion errors
//             of processed groups, the minimum-fragment filter;
//   order     kept groups by first appearance (sorted input) or by barcode
//             bytes (LSD radix over length, then 8-byte big-endian words);
//   matrix    kept in-genome records keyed (cell, position, size) and
//             radix-sorted, decoded into CSR order.
#include "common.cuh"
#include "internal.h"

#include <algorithm>

namespace sg {
namespace {

enum : uint16_t {
  F_REC = 1,        // a record (not a comment line)
  F_LEN = 2,        // end != start after the shifts
  F_GEN = 4,        // chromosome present in the genome
  F_MITO = 8,       // mitochondrial chromosome
  F_BC = 16,        // barcode present (not ".")
  F_REV = 32,       // strand "-"
  F_STRANDED = 64,  // strand column present and not "."
  F_POSERR = 128,   // position outside its chromosome
  F_FITU32 = 256,   // signed size in [0, 2^32)
  F_FITI32 = 512,   // signed size in [-2^31, 2^31)
};

constexpr int kThreads = 256;
constexpr int64_t kChunk = 64 * 1024;  // bytes of text per CTA in the line index

// ---- hashing ---------------------------------------------------------------
// SplitMix64 output function (Steele, Lea & Flood, "Fast splittable
// pseudorandom number generators", 2014), used as a 64-bit mixer.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

struct Hasher {
  uint64_t h, w;
  int nb;
  int64_t len;
  __device__ explicit Hasher(uint64_t seed) : h(mix64(seed ^ 0x6a09e667f3bcc909ull)), w(0), nb(0), len(0) {}
  __device__ __forceinline__ void push(uint8_t b) {
    w |= (uint64_t)b << (8 * nb);
    ++len;
    if (++nb == 8) {
      h = mix64(h ^ w);
      w = 0;
      nb = 0;
    }
  }
  __device__ __forceinline__ uint64_t finish() {
    if (nb) h = mix64(h ^ w);
    return mix64(h ^ ((uint64_t)len * 0x9e3779b97f4a7c15ull));
  }
};

__device__ __forceinline__ uint64_t hash_bytes(const uint8_t* p, int64_t n, uint64_t seed) {
  Hasher hs(seed);
  for (int64_t i = 0; i < n; ++i) hs.push(p[i]);
  return hs.finish();
}

// barcode location: byte offset << 16 | length (length < 65536)
__device__ __forceinline__ int64_t loc_off(uint64_t l) { return (int64_t)(l >> 16); }
__device__ __forceinline__ int loc_len(uint64_t l) { return (int)(l & 0xFFFF); }

__device__ __forceinline__ bool bytes_equal(const uint8_t* a, const uint8_t* b, int n) {
  for (int i = 0; i < n; ++i)
    if (a[i] != b[i]) return false;
  return true;
}

__device__ __forceinline__ void set_error(int* status, unsigned long long* bad, int code, int64_t line) {
  atomicCAS(status, 0, code);
  atomicMin(bad, (unsigned long long)line);
}

// ---- line index ------------------------------------------------------------
__device__ __forceinline__ int nl_in_word(uint32_t x) { return __popc(__vcmpeq4(x, 0x0a0a0a0au)) >> 3; }

__global__ void __launch_bounds__(kThreads) line_count_kernel(const uint8_t* __restrict__ text, int64_t nbytes,
                                                              int64_t* __restrict__ counts) {
  const int64_t c = blockIdx.x, b0 = c * kChunk;
  const int64_t b1 = b0 + kChunk < nbytes ? b0 + kChunk : nbytes;
  int n = 0;
  const int64_t nvec = (b1 - b0) / 16;
  const uint4* v = reinterpret_cast<const uint4*>(text + b0);
  for (int64_t i = threadIdx.x; i < nvec; i += kThreads) {
    const uint4 q = __ldg(v + i);
    n += nl_in_word(q.x) + nl_in_word(q.y) + nl_in_word(q.z) + nl_in_word(q.w);
  }
  for (int64_t p = b0 + nvec * 16 + threadIdx.x; p < b1; p += kThreads) n += text[p] == '\n';
  __shared__ int ws[kThreads / 32];
#pragma unroll
  for (int o = 16; o; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int i = 0; i < kThreads / 32; ++i) t += ws[i];
    counts[1 + c] = t;
    if (c == 0) counts[0] = 0;
  }
}

// line_start[k + 1] = 1 + position of the k-th newline; line_start[0] = 0
__global__ void __launch_bounds__(kThreads) line_fill_kernel(const uint8_t* __restrict__ text, int64_t nbytes,
                                                             const int64_t* __restrict__ before, int64_t n_lines,
                                                             int64_t* __restrict__ line_start) {
  const int64_t c = blockIdx.x, b0 = c * kChunk;
  const int64_t b1 = b0 + kChunk < nbytes ? b0 + kChunk : nbytes;
  __shared__ int wsum[kThreads / 32];
  int64_t base = before[c];  // newlines before this chunk
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t r0 = b0; r0 < b1; r0 += 16 * kThreads) {
    const int64_t p0 = r0 + 16 * (int64_t)threadIdx.x;
    uint8_t by[16];
    if (p0 + 16 <= b1) {
      const uint4 q = __ldg(reinterpret_cast<const uint4*>(text + p0));
      const uint32_t wd[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
      for (int j = 0; j < 16; ++j) by[j] = (uint8_t)(wd[j >> 2] >> (8 * (j & 3)));
    } else {
#pragma unroll
      for (int j = 0; j < 16; ++j) by[j] = p0 + j < b1 ? text[p0 + j] : 0;
    }
    int n = 0;
#pragma unroll
    for (int j = 0; j < 16; ++j) n += by[j] == '\n';
    int x = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int off = 0, tot = 0;
    for (int i = 0; i < kThreads / 32; ++i) {
      if (i < w) off += wsum[i];
      tot += wsum[i];
    }
    int64_t k = base + off + x - n;
#pragma unroll
    for (int j = 0; j < 16; ++j)
      if (by[j] == '\n') line_start[1 + k++] = p0 + j + 1;
    base += tot;
    __syncthreads();
  }
  if (c == 0 && threadIdx.x == 0) {
    line_start[0] = 0;
    // an unterminated last line ends at nbytes: its "next start" is nbytes + 1
    if (n_lines > 0 && text[nbytes - 1] != '\n') line_start[n_lines] = nbytes + 1;
  }
}

// ---- parse -----------------------------------------------------------------
struct ChromTable {
  const uint8_t* blob;    // names, concatenated, sorted by bytes
  const int64_t* off;     // n + 1 offsets into blob
  const uint64_t* size;   // chromosome length
  const uint64_t* base;   // cumulative length before the chromosome
  const uint8_t* mito;    // 1 for mitochondrial names
  const uint64_t* pk;     // first 8 bytes of each name, big-endian, zero padded
  int n;
};
constexpr int kMaxChroms = 1 << 16;

__global__ void chrom_pack(ChromTable ct, uint64_t* __restrict__ pk) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ct.n; c += gridDim.x * blockDim.x) {
    const int64_t o = ct.off[c], n = ct.off[c + 1] - o;
    uint64_t k = 0;
    for (int j = 0; j < 8; ++j) k = (k << 8) | (j < n ? ct.blob[o + j] : 0u);
    pk[c] = k;
  }
}

// Chromosome of a name given as (first 8 bytes big-endian, length, bytes).
// Names compare by bytes; (packed prefix, length) orders them the same way
// unless both names are longer than 8 bytes and share the prefix, where the
// remaining bytes decide.
__device__ int find_chrom(const ChromTable& ct, uint64_t qk, int64_t qlen, const uint8_t* q) {
  int lo = 0, hi = ct.n - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const uint64_t k = ct.pk[mid];
    const int64_t o = ct.off[mid], len = ct.off[mid + 1] - o;
    int c;
    if (qk != k) {
      c = qk < k ? -1 : 1;
    } else if (qlen > 8 && len > 8) {
      c = 0;
      const int64_t m = qlen < len ? qlen : len;
      for (int64_t j = 8; j < m && c == 0; ++j) {
        const uint8_t x = q[j], y = ct.blob[o + j];
        if (x != y) c = x < y ? -1 : 1;
      }
      if (c == 0) c = qlen < len ? -1 : (qlen > len ? 1 : 0);
    } else {
      c = qlen < len ? -1 : (qlen > len ? 1 : 0);
    }
    if (c == 0) return mid;
    if (c < 0) hi = mid - 1;
    else lo = mid + 1;
  }
  return -1;
}

__device__ __forceinline__ uint64_t sat_add(uint64_t x, int64_t s) {
  if (s >= 0) return x > UINT64_MAX - (uint64_t)s ? UINT64_MAX : x + (uint64_t)s;
  const uint64_t m = (uint64_t)(-(s + 1)) + 1;  // |s| without overflow
  return x < m ? 0 : x - m;
}

struct ParseOut {
  uint64_t* hash;
  uint64_t* loc;
  int64_t* pos;
  int64_t* val;
  uint32_t* cnt;
  uint16_t* flags;
};

// decimal digits into an unsigned accumulator; `ok` turns false on a
// non-digit or on overflow of 64 bits
__device__ __forceinline__ void push_digit(uint64_t& v, bool& ok, uint8_t c) {
  const uint32_t d = (uint32_t)c - '0';
  if (d > 9 || v > (UINT64_MAX - d) / 10) ok = false;
  else v = v * 10 + d;
}

// One pass over each line's bytes (thread per line): fields split at tabs,
// numbers accumulated and the barcode hashed as the bytes go by.  The
// kernel-wide first record and longest barcode are reduced in registers
// and per warp before one atomic each.
__global__ void __launch_bounds__(kThreads) parse_kernel(const uint8_t* __restrict__ text, int64_t nbytes,
                                                         const int64_t* __restrict__ line_start, int64_t n_lines,
                                                         ChromTable ct, int64_t shift_left, int64_t shift_right,
                                                         uint64_t seed, int bc_always, ParseOut o,
                                                         unsigned long long* first_rec,
                                                         unsigned long long* max_bc_len,
                                                         unsigned long long* bad, int* status) {
  unsigned long long my_first = ~0ull, my_bc = 0;
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n_lines; i += (int64_t)gridDim.x * kThreads) {
    const int64_t s = line_start[i];
    int64_t e = line_start[i + 1] - 1;
    if (e > nbytes) e = nbytes;
    if (e < nbytes && e > s && text[e - 1] == '\r') --e;  // CR of a CRLF line end
    if (e > s && text[s] == '#') {
      o.flags[i] = 0;
      continue;
    }
    my_first = my_first < (unsigned long long)i ? my_first : (unsigned long long)i;
    // fields 0..5: chrom, start, end, barcode, count, strand
    int f = 0;
    uint64_t ck = 0, start = 0, end = 0, cntv = 0;
    int64_t clen = 0, len1 = 0, len2 = 0, len4 = 0, bstart = s, blen = 0, slen = 0;
    bool ok1 = true, ok2 = true, ok4 = true;
    uint8_t b0 = 0, c4 = 0, sc = 0;
    Hasher hs(seed);
    for (int64_t p = s; p < e; ++p) {
      const uint8_t c = text[p];
      if (c == '\t') {
        if (++f == 6) break;
        if (f == 3) bstart = p + 1;
        continue;
      }
      switch (f) {
        case 0:
          if (clen < 8) ck |= (uint64_t)c << (56 - 8 * clen);
          ++clen;
          break;
        case 1: ++len1; push_digit(start, ok1, c); break;
        case 2: ++len2; push_digit(end, ok2, c); break;
        case 3:
          if (blen == 0) b0 = c;
          hs.push(c);
          ++blen;
          break;
        case 4:
          if (len4 == 0) c4 = c;
          ++len4;
          push_digit(cntv, ok4, c);
          break;
        default:
          sc = c;
          ++slen;
          break;
      }
    }
    const int nf = f >= 6 ? 6 : f + 1;
    bool ok = nf >= 4 && ok1 && len1 > 0 && ok2 && len2 > 0;
    uint16_t fl = F_REC;
    uint64_t count = 1;
    if (ok && nf >= 5 && !(len4 == 1 && c4 == '.')) {   // "." = 1
      ok = ok4 && len4 > 0 && !(cntv >> 32);
      count = cntv;
    }
    if (ok && nf >= 6) {
      if (slen == 1 && sc == '+') fl |= F_STRANDED;
      else if (slen == 1 && sc == '-') fl |= F_STRANDED | F_REV;
      else if (!(slen == 1 && sc == '.')) ok = false;
    }
    const bool has_bc = ok && !(blen == 1 && b0 == '.');
    if (has_bc && blen > 0xFFFF) ok = false;
    if (!ok) {
      o.flags[i] = 0;
      set_error(status, bad, SG_ERR_PARSE, i);
      continue;
    }
    // saturating shifts, preprocessing.rs:174-184
    const bool stranded = (fl & F_STRANDED) != 0;
    if (shift_left != 0) {
      start = sat_add(start, shift_left);
      if (stranded) end = sat_add(end, shift_left);
    }
    if (shift_right != 0 && !stranded) end = sat_add(end, shift_right);
    if (start != end) fl |= F_LEN;
    uint64_t h = 0, loc = 0;
    if (has_bc) {
      fl |= F_BC;
      h = hs.finish();
      loc = ((uint64_t)bstart << 16) | (uint64_t)blen;
      my_bc = my_bc > (unsigned long long)blen ? my_bc : (unsigned long long)blen;
    } else if ((fl & F_LEN) || bc_always) {
      o.flags[i] = 0;
      set_error(status, bad, SG_ERR_PARSE, i);  // a fragment without a barcode
      continue;
    }
    int64_t gpos = -1, v = 0;
    const int cid = find_chrom(ct, ck, clen, text + s);
    if (cid >= 0) {
      fl |= F_GEN;
      if (ct.mito[cid]) fl |= F_MITO;
      // import.rs:176-204 with i64 arithmetic that wraps like the release build
      const uint64_t size = end - start;
      uint64_t pp;
      if (fl & F_REV) {
        pp = end - 1;
        v = (int64_t)(0 - size);
      } else {
        pp = start;
        v = (int64_t)size;
      }
      if (pp >= ct.size[cid]) fl |= F_POSERR;
      else gpos = (int64_t)(ct.base[cid] + pp);
      if (v >= 0 && v <= (int64_t)UINT32_MAX) fl |= F_FITU32;
      if (v >= (int64_t)INT32_MIN && v <= (int64_t)INT32_MAX) fl |= F_FITI32;
    }
    o.hash[i] = h;
    o.loc[i] = loc;
    o.pos[i] = gpos;
    o.val[i] = v;
    o.cnt[i] = (uint32_t)count;
    o.flags[i] = fl;
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, my_first, off);
    const unsigned long long b = __shfl_xor_sync(0xffffffffu, my_bc, off);
    my_first = a < my_first ? a : my_first;
    my_bc = b > my_bc ? b : my_bc;
  }
  if ((threadIdx.x & 31) == 0) {
    if (my_first != ~0ull) atomicMin(first_rec, my_first);
    if (my_bc) atomicMax(max_bc_len, my_bc);
  }
}

// ---- grouping ----------------------------------------------------------------
__global__ void mark_records(int64_t n, const uint16_t* __restrict__ flags, int64_t* __restrict__ a,
                             int64_t* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint16_t f = flags[i];
    const bool rec = (f & (F_REC | F_BC)) == (F_REC | F_BC);
    a[i] = rec;
    b[i] = rec && (f & F_LEN);
  }
}

__global__ void compact_records(int64_t n, const uint16_t* __restrict__ flags, const int64_t* __restrict__ a,
                                const uint64_t* __restrict__ hash, uint64_t* __restrict__ keys,
                                uint64_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if ((flags[i] & (F_REC | F_BC)) == (F_REC | F_BC)) {
      const int64_t j = a[i] - 1;
      keys[j] = hash[i];
      vals[j] = (uint64_t)i;
    }
  }
}

__global__ void rehash_records(int64_t nrec, const uint64_t* __restrict__ vals, const uint64_t* __restrict__ loc,
                               const uint8_t* __restrict__ text, uint64_t seed, uint64_t* __restrict__ keys) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nrec; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t l = loc[vals[j]];
    keys[j] = hash_bytes(text + loc_off(l), loc_len(l), seed);
  }
}

__global__ void segment_heads(int64_t nrec, const uint64_t* __restrict__ keys, const uint64_t* __restrict__ vals,
                              const uint64_t* __restrict__ loc, const uint8_t* __restrict__ text,
                              int64_t* __restrict__ head, int* __restrict__ collide) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nrec; j += (int64_t)gridDim.x * blockDim.x) {
    bool h = j == 0 || keys[j] != keys[j - 1];
    if (!h) {
      const uint64_t a = loc[vals[j]], b = loc[vals[j - 1]];
      if (loc_len(a) != loc_len(b) || !bytes_equal(text + loc_off(a), text + loc_off(b), loc_len(a)))
        atomicExch(collide, 1);
    }
    head[j] = h;
  }
}

struct Groups {
  unsigned long long* n_all;  // records with this barcode
  unsigned long long* n_len;  // ... with end != start
  unsigned long long* uniq;   // ... in the genome, not mitochondrial
  unsigned long long* mito;   // ... in the genome, mitochondrial
  unsigned long long* total;  // sum of the count column over in-genome records
  long long* rmin;            // first / last rank among records with end != start
  long long* rmax;
  long long* err;             // lowest line with a position or size error
  int64_t* leader;            // line of the group's first record
  int64_t* cell;              // cell row, or -1
  uint8_t* wl;                // whitelisted
  int64_t* keep;              // kept flag, then its scan
};

__global__ void init_groups(int64_t G, Groups g) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G; i += (int64_t)gridDim.x * blockDim.x) {
    g.n_all[i] = g.n_len[i] = g.uniq[i] = g.mito[i] = g.total[i] = 0;
    g.rmin[i] = LLONG_MAX;
    g.rmax[i] = -1;
    g.err[i] = LLONG_MAX;
    g.cell[i] = -1;
    g.wl[i] = 0;
  }
}

// Per-group sums by warp-segmented reduction (records of a group are
// contiguous after the sort) and one atomic per run and warp.
__global__ void __launch_bounds__(kThreads) group_stats(int64_t nrec, const uint64_t* __restrict__ vals,
                                                        const int64_t* __restrict__ gid1,
                                                        const uint16_t* __restrict__ flags,
                                                        const uint32_t* __restrict__ cnt,
                                                        const int64_t* __restrict__ lrank,
                                                        const int64_t* __restrict__ val, int paired, Groups g,
                                                        unsigned long long* __restrict__ max_abs) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * kThreads;
  unsigned long long my_amax = 0;
  for (int64_t j0 = blockIdx.x * (int64_t)kThreads; j0 < nrec; j0 += stride) {
    const int64_t j = j0 + threadIdx.x;
    const bool in = j < nrec;
    int64_t gid = -1 - lane;  // distinct, negative: no run for padding lanes
    uint32_t small = 0;       // n_all | n_len << 8 | uniq << 16 | mito << 24
    unsigned long long tot = 0, amax = 0;
    long long rmn = LLONG_MAX, rmx = -1, er = LLONG_MAX;
    if (in) {
      gid = gid1[j] - 1;
      const int64_t i = (int64_t)vals[j];
      const uint16_t f = flags[i];
      const bool len = f & F_LEN, gen = len && (f & F_GEN);
      small = 1u | (len ? 1u << 8 : 0u);
      if (gen) {
        small |= (f & F_MITO) ? 1u << 24 : 1u << 16;
        tot = cnt[i];
        const bool fits = paired ? (f & F_FITU32) : (f & F_FITI32);
        if ((f & F_POSERR) || !fits) er = i;
        if (fits) {
          const int64_t v = val[i];
          amax = (unsigned long long)(v < 0 ? -v : v);
        }
      }
      if (len) rmn = rmx = lrank[i];
      if (j == 0 || gid1[j - 1] != gid1[j]) g.leader[gid] = i;
    }
    my_amax = amax > my_amax ? amax : my_amax;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t og = __shfl_down_sync(0xffffffffu, gid, o);
      const uint32_t os = __shfl_down_sync(0xffffffffu, small, o);
      const unsigned long long ot = __shfl_down_sync(0xffffffffu, tot, o);
      const long long omn = __shfl_down_sync(0xffffffffu, rmn, o);
      const long long omx = __shfl_down_sync(0xffffffffu, rmx, o);
      const long long oer = __shfl_down_sync(0xffffffffu, er, o);
      if (lane + o < 32 && og == gid) {
        small += os;
        tot += ot;
        rmn = omn < rmn ? omn : rmn;
        rmx = omx > rmx ? omx : rmx;
        er = oer < er ? oer : er;
      }
    }
    const int64_t pg = __shfl_up_sync(0xffffffffu, gid, 1);
    if (in && (lane == 0 || pg != gid)) {
      atomicAdd(g.n_all + gid, (unsigned long long)(small & 0xFF));
      if ((small >> 8) & 0xFF) atomicAdd(g.n_len + gid, (unsigned long long)((small >> 8) & 0xFF));
      if ((small >> 16) & 0xFF) atomicAdd(g.uniq + gid, (unsigned long long)((small >> 16) & 0xFF));
      if (small >> 24) atomicAdd(g.mito + gid, (unsigned long long)(small >> 24));
      if (tot) atomicAdd(g.total + gid, tot);
      if (rmx >= 0) {
        atomicMin(g.rmin + gid, rmn);
        atomicMax(g.rmax + gid, rmx);
      }
      if (er != LLONG_MAX) atomicMin(g.err + gid, er);
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, my_amax, o);
    my_amax = x > my_amax ? x : my_amax;
  }
  if (lane == 0 && my_amax) atomicMax(max_abs, my_amax);
}

// ---- whitelist ---------------------------------------------------------------
__global__ void wl_hash(int64_t W, const uint8_t* __restrict__ blob, const int64_t* __restrict__ off, uint64_t seed,
                        uint64_t* __restrict__ keys, uint64_t* __restrict__ vals) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < W; k += (int64_t)gridDim.x * blockDim.x) {
    keys[k] = hash_bytes(blob + off[k], off[k + 1] - off[k], seed);
    vals[k] = (uint64_t)k;
  }
}

__global__ void wl_lookup(int64_t G, const int64_t* __restrict__ leader, const uint64_t* __restrict__ loc,
                          const uint8_t* __restrict__ text, uint64_t seed, int64_t W,
                          const uint64_t* __restrict__ wkeys, const uint64_t* __restrict__ wvals,
                          const uint8_t* __restrict__ blob, const int64_t* __restrict__ off, uint8_t* __restrict__ wl) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < G; g += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t l = loc[leader[g]];
    const uint8_t* b = text + loc_off(l);
    const int n = loc_len(l);
    const uint64_t h = hash_bytes(b, n, seed);
    int64_t lo = 0, hi = W;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (wkeys[mid] < h) lo = mid + 1;
      else hi = mid;
    }
    uint8_t hit = 0;
    for (int64_t k = lo; k < W && wkeys[k] == h && !hit; ++k) {
      const int64_t e = (int64_t)wvals[k];
      if (off[e + 1] - off[e] == n && bytes_equal(blob + off[e], b, n)) hit = 1;
    }
    wl[g] = hit;
  }
}

// ---- decisions ---------------------------------------------------------------
__global__ void decide_groups(int64_t G, Groups g, const uint16_t* __restrict__ flags, int has_wl, int pre_min,
                              int sorted_input, uint64_t min_frag, unsigned long long* bad, int* status) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G; i += (int64_t)gridDim.x * blockDim.x) {
    bool pass = (!has_wl || g.wl[i]) && g.n_len[i] > 0;
    if (pre_min) pass = pass && g.n_all[i] >= min_frag;
    if (pass) {
      if (sorted_input && (unsigned long long)(g.rmax[i] - g.rmin[i] + 1) != g.n_len[i])
        set_error(status, bad, SG_ERR_UNSORTED, g.leader[i]);
      if (g.err[i] != LLONG_MAX) {
        const int64_t line = g.err[i];
        set_error(status, bad, (flags[line] & F_POSERR) ? SG_ERR_RANGE : SG_ERR_CONVERT, line);
      }
    }
    g.keep[i] = pass && g.uniq[i] >= min_frag;
  }
}

__global__ void kept_keys(int64_t G, const Groups g, const int64_t* __restrict__ keep_scan, int sorted_input,
                          const uint64_t* __restrict__ loc, uint64_t* __restrict__ keys, uint64_t* __restrict__ vals) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < G; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t prev = i ? keep_scan[i - 1] : 0;
    if (keep_scan[i] != prev) {
      keys[prev] = sorted_input ? (uint64_t)g.rmin[i] : (uint64_t)loc_len(loc[g.leader[i]]);
      vals[prev] = (uint64_t)i;
    }
  }
}

// big-endian 8-byte word w of each kept group's barcode, zero padded
__global__ void word_keys(int64_t K, const uint64_t* __restrict__ vals, const int64_t* __restrict__ leader,
                          const uint64_t* __restrict__ loc, const uint8_t* __restrict__ text, int w,
                          uint64_t* __restrict__ keys) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < K; r += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t l = loc[leader[vals[r]]];
    const uint8_t* b = text + loc_off(l);
    const int n = loc_len(l);
    uint64_t k = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int p = 8 * w + j;
      k = (k << 8) | (p < n ? b[p] : 0u);
    }
    keys[r] = k;
  }
}

// per cell row r (kept groups in final order): QC columns, barcode, row length
__global__ void cell_rows(int64_t K, const uint64_t* __restrict__ order, Groups g, const uint64_t* __restrict__ loc,
                          int64_t* __restrict__ row_len, uint64_t* __restrict__ bc_loc, uint64_t* __restrict__ nfrag,
                          double* __restrict__ fdup, double* __restrict__ fmito) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < K; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = (int64_t)order[r];
    g.cell[i] = r;
    const unsigned long long u = g.uniq[i], m = g.mito[i], t = g.total[i];
    row_len[r] = (int64_t)(u + m);
    bc_loc[r] = loc[g.leader[i]];
    nfrag[r] = u;
    // qc.rs:454-465, FP64 and IEEE division (0/0 gives NaN as in the reference)
    fdup[r] = 1.0 - (double)(u + m) / (double)t;
    fmito[r] = (double)m / (double)(u + m);
  }
}

__global__ void mark_matrix(int64_t nrec, const uint64_t* __restrict__ vals, const int64_t* __restrict__ gid1,
                            const int64_t* __restrict__ cell, const uint16_t* __restrict__ flags,
                            int64_t* __restrict__ m) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nrec; j += (int64_t)gridDim.x * blockDim.x) {
    const uint16_t f = flags[vals[j]];
    m[j] = cell[gid1[j] - 1] >= 0 && (f & F_LEN) && (f & F_GEN);
  }
}

struct KeyLayout {
  int vbits, pbits, rbits;
  int64_t vbias;
  bool combined;  // one 64-bit key (cell | position | size)
};

// combined: key = cell << (pbits + vbits) | pos << vbits | (val + bias);
// otherwise: k1 = val + bias, k2 = pos, k3 = cell (sorted in that order)
__global__ void matrix_keys(int64_t nrec, const uint64_t* __restrict__ vals, const int64_t* __restrict__ gid1,
                            const int64_t* __restrict__ cell, const int64_t* __restrict__ mscan,
                            const int64_t* __restrict__ pos, const int64_t* __restrict__ val, KeyLayout kl,
                            uint64_t* __restrict__ keys, uint64_t* __restrict__ slot, int64_t* __restrict__ k2,
                            int64_t* __restrict__ k3) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nrec; j += (int64_t)gridDim.x * blockDim.x) {
    const int64_t prev = j ? mscan[j - 1] : 0;
    if (mscan[j] == prev) continue;
    const int64_t i = (int64_t)vals[j];
    const uint64_t c = (uint64_t)cell[gid1[j] - 1];
    const uint64_t vb = (uint64_t)(val[i] + kl.vbias);
    const uint64_t p = (uint64_t)pos[i];
    if (kl.combined) {
      keys[prev] = (c << (kl.pbits + kl.vbits)) | (p << kl.vbits) | vb;
    } else {
      keys[prev] = vb;
      slot[prev] = (uint64_t)prev;
      k2[prev] = (int64_t)p;
      k3[prev] = (int64_t)c;
    }
  }
}

__global__ void gather_keys(int64_t n, const uint64_t* __restrict__ slot, const int64_t* __restrict__ src,
                            uint64_t* __restrict__ keys) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    keys[j] = (uint64_t)src[slot[j]];
}

__global__ void decode_combined(int64_t n, const uint64_t* __restrict__ keys, KeyLayout kl, int64_t* __restrict__ pos,
                                int32_t* __restrict__ val) {
  const uint64_t vmask = kl.vbits >= 64 ? ~0ull : ((1ull << kl.vbits) - 1);
  const uint64_t pmask = kl.pbits >= 64 ? ~0ull : ((1ull << kl.pbits) - 1);
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t k = keys[j];
    pos[j] = (int64_t)((k >> kl.vbits) & pmask);
    val[j] = (int32_t)(int64_t)((k & vmask) - (uint64_t)kl.vbias);
  }
}

__global__ void decode_slots(int64_t n, const uint64_t* __restrict__ slot, const int64_t* __restrict__ k2,
                             const uint64_t* __restrict__ vb_sorted_by_slot, int64_t vbias, int64_t* __restrict__ pos,
                             int32_t* __restrict__ val) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t s = slot[j];
    pos[j] = k2[s];
    val[j] = (int32_t)((int64_t)vb_sorted_by_slot[s] - vbias);
  }
}

__global__ void scatter_by_slot(int64_t n, const uint64_t* __restrict__ keys, const uint64_t* __restrict__ slot,
                                uint64_t* __restrict__ out) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < n; j += (int64_t)gridDim.x * blockDim.x)
    out[slot[j]] = keys[j];
}

// ---- workspace ---------------------------------------------------------------
inline int64_t al(int64_t b) { return (b + 255) / 256 * 256; }

struct Layout {
  int64_t hash, loc, pos, val, cnt, flags, a, b, head;
  int64_t k0, v0, k1, v1;            // record sort
  int64_t x0, y0, x1, y1;            // group order, then matrix sort
  int64_t wk0, wv0, wk1, wv1;        // whitelist sort
  int64_t g_all, g_len, g_uniq, g_mito, g_total, g_rmin, g_rmax, g_err, g_leader, g_cell, g_wl, g_keep;
  int64_t order, row_ptr, bc, nfrag, fdup, fmito, mscan, k2, k3, mpos, mval;
  int64_t radix, scan, scal, pk;
  int64_t total;
};

Layout frag_layout(int64_t L, int64_t W) {
  Layout y{};
  int64_t o = 0;
  auto take = [&](int64_t bytes) { const int64_t r = o; o += al(bytes < 256 ? 256 : bytes); return r; };
  const int64_t L8 = 8 * (L < 1 ? 1 : L), W8 = 8 * (W < 1 ? 1 : W);
  y.hash = take(L8); y.loc = take(L8); y.pos = take(L8); y.val = take(L8);
  y.cnt = take(4 * L); y.flags = take(2 * L); y.a = take(L8); y.b = take(L8); y.head = take(L8);
  y.k0 = take(L8); y.v0 = take(L8); y.k1 = take(L8); y.v1 = take(L8);
  y.x0 = take(L8); y.y0 = take(L8); y.x1 = take(L8); y.y1 = take(L8);
  y.wk0 = take(W8); y.wv0 = take(W8); y.wk1 = take(W8); y.wv1 = take(W8);
  y.g_all = take(L8); y.g_len = take(L8); y.g_uniq = take(L8); y.g_mito = take(L8); y.g_total = take(L8);
  y.g_rmin = take(L8); y.g_rmax = take(L8); y.g_err = take(L8); y.g_leader = take(L8); y.g_cell = take(L8);
  y.g_wl = take(L); y.g_keep = take(L8);
  y.order = take(L8); y.row_ptr = take(L8 + 8); y.bc = take(L8); y.nfrag = take(L8); y.fdup = take(L8);
  y.fmito = take(L8); y.mscan = take(L8); y.k2 = take(L8); y.k3 = take(L8); y.mpos = take(L8); y.mval = take(4 * L);
  const int64_t big = L > W ? L : W;
  y.radix = take(radix_scratch_bytes(big < 1 ? 1 : big));
  y.scan = take(scan_scratch_bytes(L + 1));
  y.scal = take(256);
  y.pk = take(8 * kMaxChroms);
  y.total = o;
  return y;
}

inline int bits_for(uint64_t maxv) {  // bits to hold values 0..maxv
  int b = 0;
  while (b < 64 && (maxv >> b)) ++b;
  return b < 1 ? 1 : b;
}

int grid_of(int64_t n) { return grid_for(n, kThreads, 8 * 152 * 8); }

// device-resident scalars in the workspace
struct Scalars {
  unsigned long long first_rec, max_bc, bad, max_abs;
  int status, collide;
};

}  // namespace
}  // namespace sg

using namespace sg;

extern "C" int64_t sg_frag_line_scratch_bytes(int64_t nbytes) {
  if (nbytes < 0) return -1;
  const int64_t nc = (nbytes + kChunk - 1) / kChunk;
  return al((nc + 1) * 8) + scan_scratch_bytes(nc + 1);
}

extern "C" int sg_frag_count_lines(const uint8_t* text, int64_t nbytes, void* scratch, int64_t* n_lines,
                                   void* stream) {
  if (nbytes < 0 || !n_lines || (nbytes > 0 && (!text || !scratch))) return SG_ERR_ARG;
  if (((uintptr_t)text & 15) != 0) return SG_ERR_ARG;
  *n_lines = 0;
  if (nbytes == 0) return SG_OK;
  cudaStream_t s = as_stream(stream);
  const int64_t nc = (nbytes + kChunk - 1) / kChunk;
  int64_t* counts = static_cast<int64_t*>(scratch);
  line_count_kernel<<<(unsigned)nc, kThreads, 0, s>>>(text, nbytes, counts);
  SG_CHECK_LAUNCH();
  if (inclusive_scan_i64(counts, nc + 1, static_cast<char*>(scratch) + al((nc + 1) * 8), s) != cudaSuccess)
    return SG_ERR_CUDA;
  int64_t nl = 0;
  uint8_t last = 0;
  if (cudaMemcpyAsync(&nl, counts + nc, 8, cudaMemcpyDeviceToHost, s) != cudaSuccess) return SG_ERR_CUDA;
  if (cudaMemcpyAsync(&last, text + nbytes - 1, 1, cudaMemcpyDeviceToHost, s) != cudaSuccess) return SG_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return SG_ERR_CUDA;
  *n_lines = nl + (last != '\n' ? 1 : 0);
  return SG_OK;
}

extern "C" int sg_frag_index_lines(const uint8_t* text, int64_t nbytes, const void* scratch, int64_t n_lines,
                                   int64_t* line_start, void* stream) {
  if (nbytes < 0 || n_lines < 0 || !line_start || (nbytes > 0 && (!text || !scratch))) return SG_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  if (nbytes == 0) {
    return cudaMemsetAsync(line_start, 0, 8, s) == cudaSuccess ? SG_OK : SG_ERR_CUDA;
  }
  const int64_t nc = (nbytes + kChunk - 1) / kChunk;
  line_fill_kernel<<<(unsigned)nc, kThreads, 0, s>>>(text, nbytes, static_cast<const int64_t*>(scratch), n_lines,
                                                     line_start);
  SG_CHECK_LAUNCH();
  return SG_OK;
}

extern "C" int64_t sg_frag_workspace_bytes(int64_t n_lines, int64_t n_whitelist) {
  if (n_lines < 0 || n_whitelist < 0) return -1;
  return frag_layout(n_lines, n_whitelist).total;
}

#define SG_CUDA(x)                                  \
  do {                                              \
    if ((x) != cudaSuccess) return SG_ERR_CUDA;     \
  } while (0)

extern "C" int sg_frag_import(const uint8_t* text, int64_t nbytes, const int64_t* line_start, int64_t n_lines,
                              const uint8_t* chrom_blob, const int64_t* chrom_off, const uint64_t* chrom_size,
                              const uint64_t* chrom_base, const uint8_t* chrom_mito, int n_chrom,
                              uint64_t genome_size, const uint8_t* wl_blob, const int64_t* wl_off, int64_t n_whitelist,
                              int has_whitelist, uint64_t min_num_fragments, int sorted_by_barcode,
                              int64_t shift_left, int64_t shift_right, uint64_t seed, void* workspace,
                              int64_t workspace_bytes, int64_t* info, void* stream) {
  if (!info || n_lines < 0 || n_chrom <= 0 || n_chrom > kMaxChroms || n_whitelist < 0 || nbytes < 0)
    return SG_ERR_ARG;
  if (n_lines > 0 && (!text || !line_start || !workspace)) return SG_ERR_ARG;
  if (!chrom_blob || !chrom_off || !chrom_size || !chrom_base || !chrom_mito) return SG_ERR_ARG;
  if (has_whitelist && n_whitelist > 0 && (!wl_blob || !wl_off)) return SG_ERR_ARG;
  if (shift_left < -(int64_t(1) << 62) || shift_left > (int64_t(1) << 62) || shift_right < -(int64_t(1) << 62) ||
      shift_right > (int64_t(1) << 62) || nbytes >= (int64_t(1) << 47))
    return SG_ERR_ARG;
  for (int i = 0; i < 10; ++i) info[i] = 0;
  info[2] = -1;
  info[3] = -1;
  if (n_lines == 0) return SG_OK;
  const Layout y = frag_layout(n_lines, n_whitelist);
  if (workspace_bytes < y.total) return SG_ERR_CAP;
  cudaStream_t s = as_stream(stream);
  char* ws = static_cast<char*>(workspace);
  int64_t nk = 0;  // kernels launched (info[8])
  auto scan_counted = [&](int64_t* d, int64_t n, void* scr, cudaStream_t st) {
    if (n > 0) nk += 3;
    return inclusive_scan_i64(d, n, scr, st);
  };
  auto sort_counted = [&](int64_t n, uint64_t* k, uint64_t* v, uint64_t* ka, uint64_t* va, int b0, int b1,
                          void* scr, cudaStream_t st, bool* alt) {
    if (n > 1 && b1 > b0) nk += 5 * ((b1 - b0 + 7) / 8);
    return radix_sort_u64(n, k, v, ka, va, b0, b1, scr, st, alt);
  };
#define LAUNCHED()   \
  do {               \
    SG_CHECK_LAUNCH(); \
    info[8] = ++nk;  \
  } while (0)
  auto P = [&](int64_t off) { return ws + off; };
  uint64_t* hash = (uint64_t*)P(y.hash);
  uint64_t* loc = (uint64_t*)P(y.loc);
  int64_t* pos = (int64_t*)P(y.pos);
  int64_t* val = (int64_t*)P(y.val);
  uint32_t* cnt = (uint32_t*)P(y.cnt);
  uint16_t* flags = (uint16_t*)P(y.flags);
  int64_t* a = (int64_t*)P(y.a);
  int64_t* b = (int64_t*)P(y.b);
  int64_t* head = (int64_t*)P(y.head);
  void* rscr = P(y.radix);
  void* sscr = P(y.scan);
  Scalars* sc = (Scalars*)P(y.scal);
  Scalars h{};
  h.first_rec = ~0ull;
  h.bad = ~0ull;
  SG_CUDA(cudaMemcpyAsync(sc, &h, sizeof(Scalars), cudaMemcpyHostToDevice, s));

  const int grid = grid_of(n_lines);
  uint64_t* pk = (uint64_t*)P(y.pk);
  ChromTable ct{chrom_blob, chrom_off, chrom_size, chrom_base, chrom_mito, pk, n_chrom};
  chrom_pack<<<(n_chrom + 255) / 256, 256, 0, s>>>(ct, pk);
  LAUNCHED();
  const int pre_min = !sorted_by_barcode && min_num_fragments > 0;
  parse_kernel<<<grid, kThreads, 0, s>>>(text, nbytes, line_start, n_lines, ct, shift_left, shift_right, seed, pre_min,
                                         ParseOut{hash, loc, pos, val, cnt, flags}, &sc->first_rec, &sc->max_bc,
                                         &sc->bad, &sc->status);
  LAUNCHED();
  mark_records<<<grid, kThreads, 0, s>>>(n_lines, flags, a, b);
  LAUNCHED();
  SG_CUDA(scan_counted(a, n_lines, sscr, s));
  SG_CUDA(scan_counted(b, n_lines, sscr, s));  // b[i] - 1 = rank among records with end != start
  int64_t nrec = 0;
  SG_CUDA(cudaMemcpyAsync(&nrec, a + n_lines - 1, 8, cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  info[4] = nrec;
  if (h.status) {
    info[3] = (int64_t)h.bad;
    { info[8] = nk; return h.status; }
  }
  if (h.first_rec == ~0ull) { info[8] = nk; return SG_OK; }  // comments only: nothing imported
  uint16_t f0 = 0;
  SG_CUDA(cudaMemcpyAsync(&f0, flags + h.first_rec, 2, cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  const int paired = (f0 & F_STRANDED) ? 0 : 1;
  info[2] = paired;
  if (nrec == 0) { info[8] = nk; return SG_OK; }

  // group records by barcode: sort by hash, check equal hashes byte for byte
  uint64_t* k0 = (uint64_t*)P(y.k0);
  uint64_t* v0 = (uint64_t*)P(y.v0);
  uint64_t* k1 = (uint64_t*)P(y.k1);
  uint64_t* v1 = (uint64_t*)P(y.v1);
  uint64_t *keys = nullptr, *vals = nullptr;
  uint64_t cur_seed = seed;
  int tries = 0;
  int64_t G = 0;
  for (;; ++tries) {
    // records in line order (so each group's first record is its earliest line)
    compact_records<<<grid, kThreads, 0, s>>>(n_lines, flags, a, hash, k0, v0);
    LAUNCHED();
    if (tries > 0) {  // a collision: the same records keyed with another seed
      cur_seed = seed + 0x9e3779b97f4a7c15ull * (uint64_t)tries;
      rehash_records<<<grid_of(nrec), kThreads, 0, s>>>(nrec, v0, loc, text, cur_seed, k0);
      LAUNCHED();
    }
    bool alt = false;
    SG_CUDA(sort_counted(nrec, k0, v0, k1, v1, 0, 64, rscr, s, &alt));
    keys = alt ? k1 : k0;
    vals = alt ? v1 : v0;
    SG_CUDA(cudaMemsetAsync(&sc->collide, 0, 4, s));
    segment_heads<<<grid_of(nrec), kThreads, 0, s>>>(nrec, keys, vals, loc, text, head, &sc->collide);
    LAUNCHED();
    SG_CUDA(scan_counted(head, nrec, sscr, s));
    int collide = 0;
    SG_CUDA(cudaMemcpyAsync(&G, head + nrec - 1, 8, cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaMemcpyAsync(&collide, &sc->collide, 4, cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaStreamSynchronize(s));
    if (!collide) break;
    if (tries >= 3) return SG_ERR_COLLISION;
  }
  info[5] = G;
  info[6] = tries;

  Groups g{(unsigned long long*)P(y.g_all), (unsigned long long*)P(y.g_len), (unsigned long long*)P(y.g_uniq),
           (unsigned long long*)P(y.g_mito), (unsigned long long*)P(y.g_total), (long long*)P(y.g_rmin),
           (long long*)P(y.g_rmax), (long long*)P(y.g_err), (int64_t*)P(y.g_leader), (int64_t*)P(y.g_cell),
           (uint8_t*)P(y.g_wl), (int64_t*)P(y.g_keep)};
  init_groups<<<grid_of(G), kThreads, 0, s>>>(G, g);
  LAUNCHED();
  group_stats<<<grid_of(nrec), kThreads, 0, s>>>(nrec, vals, head, flags, cnt, b, val, paired, g, &sc->max_abs);
  LAUNCHED();
  if (has_whitelist && n_whitelist > 0) {
    uint64_t* wk0 = (uint64_t*)P(y.wk0);
    uint64_t* wv0 = (uint64_t*)P(y.wv0);
    uint64_t* wk1 = (uint64_t*)P(y.wk1);
    uint64_t* wv1 = (uint64_t*)P(y.wv1);
    wl_hash<<<grid_of(n_whitelist), kThreads, 0, s>>>(n_whitelist, wl_blob, wl_off, cur_seed, wk0, wv0);
    LAUNCHED();
    bool alt = false;
    SG_CUDA(sort_counted(n_whitelist, wk0, wv0, wk1, wv1, 0, 64, rscr, s, &alt));
    wl_lookup<<<grid_of(G), kThreads, 0, s>>>(G, g.leader, loc, text, cur_seed, n_whitelist, alt ? wk1 : wk0,
                                              alt ? wv1 : wv0, wl_blob, wl_off, g.wl);
    LAUNCHED();
  }
  decide_groups<<<grid_of(G), kThreads, 0, s>>>(G, g, flags, has_whitelist, pre_min, sorted_by_barcode,
                                                min_num_fragments, &sc->bad, &sc->status);
  LAUNCHED();
  SG_CUDA(scan_counted(g.keep, G, sscr, s));
  int64_t K = 0;
  SG_CUDA(cudaMemcpyAsync(&K, g.keep + G - 1, 8, cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  if (h.status) {
    info[3] = (int64_t)h.bad;
    { info[8] = nk; return h.status; }
  }
  info[0] = K;
  if (K == 0) { info[8] = nk; return SG_OK; }

  // order the kept groups: first appearance, or barcode bytes
  uint64_t* x0 = (uint64_t*)P(y.x0);
  uint64_t* y0 = (uint64_t*)P(y.y0);
  uint64_t* x1 = (uint64_t*)P(y.x1);
  uint64_t* y1 = (uint64_t*)P(y.y1);
  kept_keys<<<grid_of(G), kThreads, 0, s>>>(G, g, g.keep, sorted_by_barcode, loc, x0, y0);
  LAUNCHED();
  uint64_t *ok = x0, *ov = y0, *ak = x1, *av = y1;
  auto sort_kv = [&](int bits) -> int {
    bool alt = false;
    if (sort_counted(K, ok, ov, ak, av, 0, bits, rscr, s, &alt) != cudaSuccess) return SG_ERR_CUDA;
    if (alt) {
      std::swap(ok, ak);
      std::swap(ov, av);
    }
    return SG_OK;
  };
  if (sorted_by_barcode) {
    if (int e = sort_kv(bits_for((uint64_t)n_lines))) return e;
  } else {
    if (int e = sort_kv(bits_for(h.max_bc))) return e;
    for (int w = (int)((h.max_bc + 7) / 8) - 1; w >= 0; --w) {
      word_keys<<<grid_of(K), kThreads, 0, s>>>(K, ov, g.leader, loc, text, w, ok);
      LAUNCHED();
      if (int e = sort_kv(64)) return e;
    }
  }
  uint64_t* order = (uint64_t*)P(y.order);
  SG_CUDA(cudaMemcpyAsync(order, ov, K * 8, cudaMemcpyDeviceToDevice, s));
  int64_t* row_ptr = (int64_t*)P(y.row_ptr);
  SG_CUDA(cudaMemsetAsync(row_ptr, 0, 8, s));
  cell_rows<<<grid_of(K), kThreads, 0, s>>>(K, order, g, loc, row_ptr + 1, (uint64_t*)P(y.bc), (uint64_t*)P(y.nfrag),
                                            (double*)P(y.fdup), (double*)P(y.fmito));
  LAUNCHED();
  SG_CUDA(scan_counted(row_ptr + 1, K, sscr, s));

  // the matrix: kept in-genome records sorted by (cell, position, size)
  int64_t* mscan = (int64_t*)P(y.mscan);
  mark_matrix<<<grid_of(nrec), kThreads, 0, s>>>(nrec, vals, head, g.cell, flags, mscan);
  LAUNCHED();
  SG_CUDA(scan_counted(mscan, nrec, sscr, s));
  int64_t nnz = 0;
  SG_CUDA(cudaMemcpyAsync(&nnz, mscan + nrec - 1, 8, cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaMemcpyAsync(&h, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, s));
  SG_CUDA(cudaStreamSynchronize(s));
  info[1] = nnz;
  if (nnz == 0) { info[8] = nk; return SG_OK; }
  KeyLayout kl{};
  const uint64_t amax = h.max_abs;
  kl.vbias = paired ? 0 : (int64_t)amax;
  kl.vbits = bits_for(paired ? amax : 2 * amax);
  kl.pbits = bits_for(genome_size > 0 ? genome_size - 1 : 0);
  kl.rbits = bits_for((uint64_t)(K - 1));
  kl.combined = kl.vbits + kl.pbits + kl.rbits <= 64;
  info[7] = kl.combined ? 0 : 1;
  int64_t* k2 = (int64_t*)P(y.k2);
  int64_t* k3 = (int64_t*)P(y.k3);
  int64_t* mpos = (int64_t*)P(y.mpos);
  int32_t* mval = (int32_t*)P(y.mval);
  matrix_keys<<<grid_of(nrec), kThreads, 0, s>>>(nrec, vals, head, g.cell, mscan, pos, val, kl, x0, y0, k2, k3);
  LAUNCHED();
  if (kl.combined) {
    bool alt = false;
    SG_CUDA(sort_counted(nnz, x0, nullptr, x1, nullptr, 0, kl.vbits + kl.pbits + kl.rbits, rscr, s, &alt));
    decode_combined<<<grid_of(nnz), kThreads, 0, s>>>(nnz, alt ? x1 : x0, kl, mpos, mval);
    LAUNCHED();
  } else {
    // LSD over three keys with the slot as payload: size, then position, then cell
    uint64_t *ck = x0, *cv = y0, *dk = x1, *dv = y1;
    bool alt = false;
    SG_CUDA(sort_counted(nnz, ck, cv, dk, dv, 0, kl.vbits, rscr, s, &alt));
    if (alt) { std::swap(ck, dk); std::swap(cv, dv); }
    // remember each slot's biased size before the keys are overwritten
    uint64_t* vb_by_slot = (uint64_t*)P(y.order);  // order is no longer needed (cells are assigned)
    scatter_by_slot<<<grid_of(nnz), kThreads, 0, s>>>(nnz, ck, cv, vb_by_slot);
    LAUNCHED();
    gather_keys<<<grid_of(nnz), kThreads, 0, s>>>(nnz, cv, k2, ck);
    LAUNCHED();
    SG_CUDA(sort_counted(nnz, ck, cv, dk, dv, 0, kl.pbits, rscr, s, &alt));
    if (alt) { std::swap(ck, dk); std::swap(cv, dv); }
    gather_keys<<<grid_of(nnz), kThreads, 0, s>>>(nnz, cv, k3, ck);
    LAUNCHED();
    SG_CUDA(sort_counted(nnz, ck, cv, dk, dv, 0, kl.rbits, rscr, s, &alt));
    if (alt) { std::swap(ck, dk); std::swap(cv, dv); }
    decode_slots<<<grid_of(nnz), kThreads, 0, s>>>(nnz, cv, k2, vb_by_slot, kl.vbias, mpos, mval);
    LAUNCHED();
  }
  SG_CUDA(cudaStreamSynchronize(s));
  info[8] = nk;
  return SG_OK;
}
#undef LAUNCHED

extern "C" int sg_frag_emit(const void* workspace, int64_t n_lines, int64_t n_whitelist, const int64_t* info,
                            int64_t* out_indptr, int64_t* out_indices, int32_t* out_data, uint64_t* out_bc_loc,
                            uint64_t* out_n_fragment, double* out_frac_dup, double* out_frac_mito, void* stream) {
  if (!workspace || !info || n_lines < 0 || n_whitelist < 0) return SG_ERR_ARG;
  const int64_t K = info[0], nnz = info[1];
  if (K <= 0) return SG_OK;
  if (!out_indptr || !out_bc_loc || !out_n_fragment || !out_frac_dup || !out_frac_mito) return SG_ERR_ARG;
  if (nnz > 0 && (!out_indices || !out_data)) return SG_ERR_ARG;
  const Layout y = frag_layout(n_lines, n_whitelist);
  const char* ws = static_cast<const char*>(workspace);
  cudaStream_t s = as_stream(stream);
  SG_CUDA(cudaMemcpyAsync(out_indptr, ws + y.row_ptr, (K + 1) * 8, cudaMemcpyDeviceToDevice, s));
  SG_CUDA(cudaMemcpyAsync(out_bc_loc, ws + y.bc, K * 8, cudaMemcpyDeviceToDevice, s));
  SG_CUDA(cudaMemcpyAsync(out_n_fragment, ws + y.nfrag, K * 8, cudaMemcpyDeviceToDevice, s));
  SG_CUDA(cudaMemcpyAsync(out_frac_dup, ws + y.fdup, K * 8, cudaMemcpyDeviceToDevice, s));
  SG_CUDA(cudaMemcpyAsync(out_frac_mito, ws + y.fmito, K * 8, cudaMemcpyDeviceToDevice, s));
  if (nnz > 0) {
    SG_CUDA(cudaMemcpyAsync(out_indices, ws + y.mpos, nnz * 8, cudaMemcpyDeviceToDevice, s));
    SG_CUDA(cudaMemcpyAsync(out_data, ws + y.mval, nnz * 4, cudaMemcpyDeviceToDevice, s));
  }
  return SG_OK;
}
