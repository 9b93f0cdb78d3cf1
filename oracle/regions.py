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
