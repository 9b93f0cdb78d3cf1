"""ORACLE (test infrastructure only): cell-by-region counts restated in Python.

Restates ``snap.pp.make_peak_matrix`` over fragments
(snapatac2-core/src/feature_count/matrix.rs:95-170) loop for loop:

* fragments come from ``obsm['fragment_paired']`` / ``['fragment_single']``
  as ``pair_to_fragments`` / ``single_to_fragments`` rebuild them
  (snapatac2-core/src/feature_count/data_iter.rs:27-117): paired rows give
  [start, start + size) after the size filters; single-end rows give a 1 bp
  read at the stored position;
* ``RegionCounter::insert_fragment`` (snapatac2-core/src/feature_count/counter.rs:117-146):
  single-end reads and the "insertion" strategy add 1 to every region that
  overlaps each insertion ([start, start + 1) and [end - 1, end)),
  "fragment" adds 1 to every region overlapping the whole fragment,
  "paired-insertion" adds 1 once to every region hit by either insertion;
* regions: the peaks in input order with repeats dropped (the bed-utils
  0.7.1 ``GIntervalIndexSet``, an index set of intervals; third-party, not in
  the reference tree), overlap = half-open intersection on the same
  chromosome; row entries sorted by region index (``get_values`` iterates a
  ``BTreeMap``);
* peak strings "chrom:start-end" (``GenomicRange::from_str``), feature names
  the same form (``pretty_show``).
"""
from __future__ import annotations

import numpy as np


def parse_region(s: str) -> tuple[str, int, int]:
    chrom, rng = s.strip().rsplit(":", 1)
    a, b = rng.split("-")
    return chrom, int(a), int(b)


def unique_regions(peaks) -> list[tuple[str, int, int]]:
    seen, out = set(), []
    for p in peaks:
        r = parse_region(p) if isinstance(p, str) else tuple(p)
        if r not in seen:
            seen.add(r)
            out.append(r)
    return out


def region_counts(indptr, pos, length, chrom_names, chrom_sizes, peaks, *, strategy="paired-insertion",
                  paired=True, min_frag_size=None, max_frag_size=None):
    """CSR (indptr, indices, data) of the cell-by-region count matrix and the
    feature names."""
    regions = unique_regions(peaks)
    starts = np.concatenate([[0], np.cumsum(np.asarray(chrom_sizes, dtype=np.int64))])
    by_chrom: dict = {}
    for k, (c, s, e) in enumerate(regions):
        by_chrom.setdefault(c, []).append((s, e, k))
    arrays = {c: (np.array([v[0] for v in lst], dtype=np.int64), np.array([v[1] for v in lst], dtype=np.int64),
                  np.array([v[2] for v in lst], dtype=np.int64)) for c, lst in by_chrom.items()}

    def hits(c, qs, qe):
        if c not in arrays:
            return []
        rs, re_, rk = arrays[c]
        return sorted(rk[(rs < qe) & (re_ > qs)].tolist())

    indptr = np.asarray(indptr, dtype=np.int64)
    pos = np.asarray(pos, dtype=np.int64)
    out_ptr = [0]
    out_idx, out_val = [], []
    for r in range(indptr.size - 1):
        counts: dict = {}
        for j in range(indptr[r], indptr[r + 1]):
            p = int(pos[j])
            ci = int(np.searchsorted(starts, p, side="right") - 1)
            if ci >= len(chrom_names):
                raise ValueError(f"position {p} outside the genome")
            c = chrom_names[ci]
            s = p - int(starts[ci])
            if not paired:
                hs = hits(c, s, s + 1)
            else:
                size = int(length[j])
                if min_frag_size is not None and size < min_frag_size:
                    continue
                if max_frag_size is not None and size > max_frag_size:
                    continue
                e = s + size
                if strategy == "fragment":
                    hs = hits(c, s, e)
                elif strategy == "insertion":
                    hs = hits(c, s, s + 1) + hits(c, e - 1, e)
                else:
                    hs = sorted(set(hits(c, s, s + 1)) | set(hits(c, e - 1, e)))
            for k in hs:
                counts[k] = counts.get(k, 0) + 1
        for k in sorted(counts):
            out_idx.append(k)
            out_val.append(counts[k])
        out_ptr.append(len(out_idx))
    names = [f"{c}:{s}-{e}" for c, s, e in regions]
    return (np.array(out_ptr, dtype=np.int64), np.array(out_idx, dtype=np.int64),
            np.array(out_val, dtype=np.uint32), names)


_STRATEGY_CODES = {"insertion": 0, "fragment": 1, "paired-insertion": 2}


def region_counts_c(indptr, pos, length, chrom_names, chrom_sizes, peaks, *, strategy="paired-insertion",
                    paired=True, min_frag_size=None, max_frag_size=None, n_threads: int = 0, timing=None):
    """``region_counts`` through oracle/regions.c (OpenMP over cells; same
    result tuple).  Regions on chromosomes outside the genome stay features
    that no fragment hits.  ``timing`` (a dict) receives ``count_s``, the
    seconds of the two counting passes without the region index set-up."""
    import ctypes
    import time
    from ._build import load_lib
    lib = load_lib("regions")
    f = lib.oracle_region_counts
    P, I64 = ctypes.c_void_p, ctypes.c_int64
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, I64, P, P, P, ctypes.c_int, P, P, P, P, P, P, ctypes.c_int, I64, I64, ctypes.c_int,
                  P, P, P, P]
    regions = unique_regions(peaks)
    cid = {c: i for i, c in enumerate(chrom_names)}
    rows = sorted((cid[c], s, e, k) for k, (c, s, e) in enumerate(regions) if c in cid)
    nc = len(chrom_names)
    a = np.array(rows, dtype=np.int64).reshape(-1, 4)
    rptr = np.zeros(nc + 1, dtype=np.int64)
    np.cumsum(np.bincount(a[:, 0], minlength=nc), out=rptr[1:])
    rstart, rend, rid = (np.ascontiguousarray(a[:, i]) for i in (1, 2, 3))
    rmax = rend.copy()
    for c in range(nc):
        if rptr[c + 1] > rptr[c]:
            rmax[rptr[c]:rptr[c + 1]] = np.maximum.accumulate(rend[rptr[c]:rptr[c + 1]])
    cstart = np.concatenate([[0], np.cumsum(np.asarray(chrom_sizes, dtype=np.uint64))]).astype(np.uint64)
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    pos = np.ascontiguousarray(pos, dtype=np.uint64)
    n = indptr.size - 1
    code = _STRATEGY_CODES[strategy] if paired else 3
    ln = np.ascontiguousarray(length, dtype=np.uint32) if paired else None
    mn = -1 if min_frag_size is None else int(min_frag_size)
    mx = -1 if max_frag_size is None else int(max_frag_size)
    out_ptr = np.zeros(n + 1, dtype=np.int64)
    bad = ctypes.c_int64(-1)
    ptrs = lambda x: None if x is None else x.ctypes.data  # noqa: E731
    args = [n, ptrs(indptr), ptrs(pos), ptrs(ln), nc, ptrs(cstart), ptrs(rptr), ptrs(rstart), ptrs(rend), ptrs(rmax),
            ptrs(rid), code, mn, mx, int(n_threads)]
    t0 = time.perf_counter()
    err = f(0, *args, ptrs(out_ptr), None, None, ctypes.byref(bad))
    if err == 2:
        raise ValueError(f"position {int(pos[bad.value])} outside the genome (fragment {bad.value})")
    if err:
        raise RuntimeError(f"oracle_region_counts failed ({err})")
    np.cumsum(out_ptr, out=out_ptr)
    out_idx = np.empty(max(int(out_ptr[-1]), 1), dtype=np.int64)
    out_val = np.empty(max(int(out_ptr[-1]), 1), dtype=np.uint32)
    err = f(1, *args, ptrs(out_ptr), ptrs(out_idx), ptrs(out_val), ctypes.byref(bad))
    if err:
        raise RuntimeError(f"oracle_region_counts failed ({err})")
    if timing is not None:
        timing["count_s"] = time.perf_counter() - t0
    nnz = int(out_ptr[-1])
    names = [f"{c}:{s}-{e}" for c, s, e in regions]
    return out_ptr, out_idx[:nnz], out_val[:nnz], names


def aggregate_x(X, var_names, chrom_names, peaks):
    """``use_x=True`` of ``create_peak_matrix`` (snapatac2-core/src/feature_count/matrix.rs:121-128):
    ``read_chrom_values().aggregate_by(RegionCounter)`` (data_iter.rs:866-891)
    -- each entry (feature interval j, value v) of a cell's row adds v to
    every region overlapping interval j (``RegionCounter::insert``,
    counter.rs:95-106); rows sorted by region index.  Returns (indptr,
    indices, data as float64, names)."""
    import scipy.sparse as sp
    X = sp.csr_matrix(X)
    regions = unique_regions(peaks)
    by_chrom: dict = {}
    for k, (c, s, e) in enumerate(regions):
        by_chrom.setdefault(c, []).append((s, e, k))
    arrays = {c: (np.array([v[0] for v in lst], dtype=np.int64), np.array([v[1] for v in lst], dtype=np.int64),
                  np.array([v[2] for v in lst], dtype=np.int64)) for c, lst in by_chrom.items()}
    feat = [parse_region(str(v)) for v in var_names]
    hit_of = []
    for c, s, e in feat:
        if c in arrays:
            rs, re_, rk = arrays[c]
            hit_of.append(sorted(rk[(rs < e) & (re_ > s)].tolist()))
        else:
            hit_of.append([])
    out_ptr, out_idx, out_val = [0], [], []
    for r in range(X.shape[0]):
        acc: dict = {}
        for j, v in zip(X.indices[X.indptr[r]:X.indptr[r + 1]], X.data[X.indptr[r]:X.indptr[r + 1]]):
            for k in hit_of[int(j)]:
                acc[k] = acc.get(k, 0.0) + float(v)
        for k in sorted(acc):
            out_idx.append(k)
            out_val.append(acc[k])
        out_ptr.append(len(out_idx))
    names = [f"{c}:{s}-{e}" for c, s, e in regions]
    return (np.array(out_ptr, dtype=np.int64), np.array(out_idx, dtype=np.int64),
            np.array(out_val, dtype=np.float64), names)
