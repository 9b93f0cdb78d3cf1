"""ORACLE -- test infrastructure only.

Tile binning restated twice, so that the two restatements check each other:

* ``tile_bin``        calls ``tile_bin.c`` (OpenMP, per-row sort + run-length,
                      restating ``gen_mat_pair``, ``data_iter.rs:347-415``);
* ``tile_bin_numpy``  vectorised NumPy version of the same arithmetic.

Both take the reference's ``fragment_paired`` encoding (row pointer, global
start index, length) and return a CSR matrix (int64 indptr, int32 tile
index, uint32 count) with sorted, unique tile indices per row, exactly what
``to_csr_data`` produces in the reference.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._build import load_lib

STRATEGIES = {"insertion": 0, "fragment": 1, "paired-insertion": 2, "single": 3}


class OracleError(RuntimeError):
    def __init__(self, code: int, entry: int):
        super().__init__(f"oracle tile binning failed with status {code} at entry {entry}")
        self.code = code
        self.entry = entry


def _exclude_mask(chrom_sizes, exclude_chroms) -> np.ndarray:
    names = [n for n, _ in chrom_sizes]
    ex = set(exclude_chroms or [])
    return np.array([1 if n in ex else 0 for n in names], dtype=np.uint8)


def tile_bin(indptr, pos, length, chrom_sizes, *, bin_size=500, exclude_chroms=("chrM", "chrY", "M", "Y"),
             counting_strategy="paired-insertion", min_frag_size=None, max_frag_size=None):
    lib = load_lib("tilebin")
    f = lib.oracle_tile_bin
    f.restype = ctypes.c_int64
    P = ctypes.c_void_p
    f.argtypes = [P, ctypes.c_int64, P, P, P, P, ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                  ctypes.c_int64, ctypes.c_int64, P, P, P, ctypes.c_int64, P]
    indptr = np.ascontiguousarray(indptr, dtype=np.int64)
    pos = np.ascontiguousarray(pos, dtype=np.uint64)
    length = np.ascontiguousarray(length, dtype=np.uint32)
    clen = np.ascontiguousarray([s for _, s in chrom_sizes], dtype=np.uint64)
    excl = _exclude_mask(chrom_sizes, exclude_chroms)
    n = indptr.shape[0] - 1
    out_ptr = np.zeros(n + 1, dtype=np.int64)
    bad = np.zeros(1, dtype=np.int64)
    st = STRATEGIES[counting_strategy]
    mn = -1 if min_frag_size is None else int(min_frag_size)
    mx = -1 if max_frag_size is None else int(max_frag_size)
    args = [indptr.ctypes.data, n, pos.ctypes.data, length.ctypes.data, clen.ctypes.data,
            excl.ctypes.data, len(clen), int(bin_size), st, mn, mx]
    nnz = f(*args, out_ptr.ctypes.data, None, None, 0, bad.ctypes.data)
    if nnz < 0:
        raise OracleError(int(-nnz), int(bad[0]))
    idx = np.empty(nnz, dtype=np.int32)
    cnt = np.empty(nnz, dtype=np.uint32)
    r = f(*args, out_ptr.ctypes.data, idx.ctypes.data, cnt.ctypes.data, nnz, bad.ctypes.data)
    if r < 0:
        raise OracleError(int(-r), int(bad[0]))
    lib.oracle_tile_ncols.restype = ctypes.c_uint64
    lib.oracle_tile_ncols.argtypes = [P, P, ctypes.c_int, ctypes.c_uint64]
    ncols = int(lib.oracle_tile_ncols(clen.ctypes.data, excl.ctypes.data, len(clen), int(bin_size)))
    return out_ptr, idx, cnt, ncols


def tile_bin_numpy(indptr, pos, length, chrom_sizes, *, bin_size=500,
                   exclude_chroms=("chrM", "chrY", "M", "Y"), counting_strategy="paired-insertion",
                   min_frag_size=None, max_frag_size=None):
    """Vectorised restatement of ``gen_mat_pair`` / ``gen_mat_single``."""
    indptr = np.asarray(indptr, dtype=np.int64)
    pos = np.asarray(pos, dtype=np.uint64)
    length = np.asarray(length, dtype=np.uint64)
    sizes = np.array([s for _, s in chrom_sizes], dtype=np.uint64)
    excl = _exclude_mask(chrom_sizes, exclude_chroms).astype(bool)
    base_end = np.cumsum(sizes, dtype=np.uint64)
    nbins = (sizes + np.uint64(bin_size - 1)) // np.uint64(bin_size)
    nbins_kept = np.where(excl, np.uint64(0), nbins)
    bin_off = np.concatenate([[0], np.cumsum(nbins_kept)[:-1]]).astype(np.uint64)
    n = indptr.shape[0] - 1
    row = np.repeat(np.arange(n, dtype=np.int64), np.diff(indptr))
    c = np.searchsorted(base_end, pos, side="right")
    if np.any(c >= len(sizes)):
        raise OracleError(2, int(np.flatnonzero(c >= len(sizes))[0]))
    start = pos - np.where(c > 0, base_end[np.maximum(c - 1, 0)], np.uint64(0))
    keep = ~excl[c]
    strategy = counting_strategy
    if strategy != "single":
        with np.errstate(over="ignore"):
            end = start + length - np.uint64(1)
        if min_frag_size is not None:
            keep &= length >= np.uint64(min_frag_size)
        if max_frag_size is not None:
            keep &= length <= np.uint64(max_frag_size)
        bad = keep & (end >= sizes[c])
        if np.any(bad):
            raise OracleError(2, int(np.flatnonzero(bad)[0]))
    row, c, start = row[keep], c[keep], start[keep]
    lo = (bin_off[c] + start // np.uint64(bin_size)).astype(np.int64)
    if strategy == "single":
        keys_r, keys_b = row, lo
    else:
        end = end[keep]
        hi = (bin_off[c] + end // np.uint64(bin_size)).astype(np.int64)
        if strategy == "insertion":
            keys_r = np.concatenate([row, row])
            keys_b = np.concatenate([lo, hi])
        elif strategy == "paired-insertion":
            two = hi != lo
            keys_r = np.concatenate([row, row[two]])
            keys_b = np.concatenate([lo, hi[two]])
        elif strategy == "fragment":
            span = np.maximum(hi - lo + 1, 0)
            keys_r = np.repeat(row, span)
            first = np.repeat(lo, span)
            offs = np.arange(int(span.sum()), dtype=np.int64) - np.repeat(np.cumsum(span) - span, span)
            keys_b = first + offs
        else:
            raise ValueError(strategy)
    key = (keys_r << np.int64(32)) | keys_b
    uk, cnt = np.unique(key, return_counts=True)
    r = uk >> np.int64(32)
    out_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=out_ptr[1:])
    return out_ptr, (uk & np.int64(0xFFFFFFFF)).astype(np.int32), cnt.astype(np.uint32), int(nbins_kept.sum())
