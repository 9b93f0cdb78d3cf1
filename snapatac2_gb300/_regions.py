"""``snap.pp.make_peak_matrix`` on the GPU: cell-by-region counts.

Drop-in counterpart of ``snapatac2-python/python/snapatac2/preprocessing/_basic.py:577-705``
over the PyO3 ``mk_peak_matrix`` (``snapatac2-python/src/preprocessing.rs:370-430``)
and ``create_peak_matrix`` (``snapatac2-core/src/feature_count/matrix.rs:95-170``).
Region lookup and counting run in ``csrc/region_count.cu`` behind the C ABI
(``sg_region_plan`` / ``sg_region_run`` / ``sg_tile_emit``).
"""
from __future__ import annotations

import ctypes
import gzip
from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from ._anndata import AnnData
from ._binning import STRATEGIES, DeviceCSR


def parse_region(s: str) -> tuple[str, int, int]:
    """``GenomicRange::from_str`` ("chrom:start-end", bed-utils 0.7.1)."""
    chrom, rng = s.strip().rsplit(":", 1)
    a, b = rng.split("-")
    return chrom, int(a), int(b)


@dataclass
class RegionSet:
    """Regions on the device, grouped by chromosome and sorted by start."""
    names: list          # feature names in feature order ("chrom:start-end")
    ptr: torch.Tensor    # int64 [n_chrom + 1]
    start: torch.Tensor  # int64 (uint64 bits)
    end: torch.Tensor
    maxend: torch.Tensor
    rid: torch.Tensor    # int32 (uint32 bits): feature index


def build_regions(peaks, chrom_names: list, device) -> RegionSet:
    """Feature list of ``peaks`` (strings or (chrom, start, end) tuples) with
    repeats dropped, first occurrence kept (the index set of intervals of
    ``create_peak_matrix``); regions on chromosomes outside the genome are
    features that no fragment can hit."""
    seen, regions = set(), []
    for p in peaks:
        r = parse_region(p) if isinstance(p, str) else (str(p[0]), int(p[1]), int(p[2]))
        if r not in seen:
            seen.add(r)
            regions.append(r)
    cid = {c: i for i, c in enumerate(chrom_names)}
    rows = [(cid[c], s, e, k) for k, (c, s, e) in enumerate(regions) if c in cid]
    nc = len(chrom_names)
    if rows:
        a = np.array(rows, dtype=np.int64)
        order = np.lexsort((a[:, 1], a[:, 0]))
        a = a[order]
        ch, st, en, k = a[:, 0], a[:, 1], a[:, 2], a[:, 3]
    else:
        ch = st = en = k = np.zeros(0, dtype=np.int64)
    ptr = np.zeros(nc + 1, dtype=np.int64)
    np.cumsum(np.bincount(ch, minlength=nc), out=ptr[1:])
    mx = en.copy()
    for c in range(nc):
        if ptr[c + 1] > ptr[c]:
            mx[ptr[c]:ptr[c + 1]] = np.maximum.accumulate(en[ptr[c]:ptr[c + 1]])
    t = lambda x, dt: torch.from_numpy(np.ascontiguousarray(x.astype(dt))).to(device)  # noqa: E731
    names = [f"{c}:{s}-{e}" for c, s, e in regions]
    return RegionSet(names, t(ptr, np.int64), t(st, np.int64), t(en, np.int64), t(mx, np.int64),
                     t(k, np.int32))


def region_matrix(indptr: torch.Tensor, pos: torch.Tensor, length: torch.Tensor | None, chrom_sizes,
                  regions: RegionSet, *, strategy: str, exclude=None, min_frag_size=None,
                  max_frag_size=None) -> DeviceCSR:
    """Cell-by-region counts of fragments resident on the GPU (``strategy``:
    "insertion", "fragment", "paired-insertion" for paired data, "single")."""
    L = _lib.lib()
    dev = indptr.device
    n = int(indptr.shape[0] - 1)
    F = int(pos.shape[0])
    st = STRATEGIES[strategy]
    names = list(chrom_sizes.names)
    chrom_end = torch.from_numpy(np.cumsum(np.asarray(chrom_sizes.sizes, dtype=np.uint64)).view(np.int64)).to(dev)
    excl = torch.tensor([1 if c in (exclude or ()) else 0 for c in names], dtype=torch.uint8, device=dev)
    if length is None:
        length = torch.zeros(max(F, 1), dtype=torch.int32, device=dev)
    mn = -1 if min_frag_size is None else int(min_frag_size)
    mx = -1 if max_frag_size is None else int(max_frag_size)
    nf = len(regions.names)
    sh = torch.cuda.current_stream(dev).cuda_stream
    status = _lib.DeviceStatus(dev)
    key_ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    scan_scr = torch.empty(int(L.sg_scan_scratch_bytes(n + 1)), dtype=torch.uint8, device=dev)
    rargs = [chrom_end.data_ptr(), excl.data_ptr(), len(names), regions.ptr.data_ptr(),
             regions.start.data_ptr() if regions.start.numel() else None,
             regions.end.data_ptr() if regions.end.numel() else None,
             regions.maxend.data_ptr() if regions.maxend.numel() else None,
             regions.rid.data_ptr() if regions.rid.numel() else None, nf, st, mn, mx]
    _lib.check(L.sg_region_plan(indptr.data_ptr(), n, F, pos.data_ptr(), length.data_ptr(), *rargs,
                                key_ptr.data_ptr(), scan_scr.data_ptr(), status.status_ptr, status.bad_ptr, sh),
               "sg_region_plan")
    status.raise_if_error("peak matrix: fragment position outside the genome", "fragment")
    K = int(key_ptr[n].item()) if n > 0 else 0
    nbytes = int(L.sg_tile_scratch_bytes(K))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
    out_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    _lib.check(L.sg_region_run(indptr.data_ptr(), n, F, pos.data_ptr(), length.data_ptr(), *rargs,
                               key_ptr.data_ptr(), scratch.data_ptr(), nbytes, out_indptr.data_ptr(),
                               scan_scr.data_ptr(), status.status_ptr, status.bad_ptr, sh), "sg_region_run")
    status.raise_if_error("peak matrix")
    nnz = int(out_indptr[n].item()) if n > 0 else 0
    out_idx = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    out_cnt = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    _lib.check(L.sg_tile_emit(n, key_ptr.data_ptr(), scratch.data_ptr(), nbytes, out_indptr.data_ptr(),
                              out_idx.data_ptr(), out_cnt.data_ptr(), nnz, status.status_ptr, sh), "sg_tile_emit")
    status.raise_if_error("peak matrix (emit)")
    return DeviceCSR(out_indptr, out_idx[:nnz], out_cnt[:nnz], (n, nf))


def _peaks_from(adata, use_rep, peak_file):
    if peak_file is not None and use_rep is not None:
        raise RuntimeError("'peak_file' and 'use_rep' cannot be both set")
    if use_rep is None and peak_file is None:
        use_rep = "peaks"
    if peak_file is not None:
        opener = gzip.open if str(peak_file).endswith(".gz") else open
        with opener(peak_file, "rt") as f:
            return [line.strip() for line in f]
    if isinstance(use_rep, str):
        df = adata.uns[use_rep]
        if hasattr(df, "columns"):
            return list(df[df.columns[0]])
        if isinstance(df, dict):
            return list(next(iter(df.values())))
        return list(df)
    return list(use_rep)


def _feature_intervals(var_names):
    """(chrom names, chrom id per feature, start, end) of X's features: from
    the tile layout of a tile matrix (no strings), else by parsing
    "chrom:start-end" names (``GenomicRange::from_str``)."""
    from .genome import TileNames
    if isinstance(var_names, TileNames):
        gi = var_names._index
        counts = np.diff(np.concatenate([[0], gi.binned_accum.astype(np.int64)]))
        cid = np.repeat(np.arange(len(gi.names), dtype=np.int64), counts)
        first = np.repeat(np.concatenate([[0], gi.binned_accum[:-1].astype(np.int64)]), counts)
        start = (np.arange(int(counts.sum()), dtype=np.int64) - first) * gi.step
        end = np.minimum(start + gi.step, np.asarray(gi.sizes, dtype=np.int64)[cid])
        return list(gi.names), cid, start, end
    names, table, cid, start, end = [], {}, [], [], []
    for v in var_names:
        c, a, b = parse_region(str(v))
        if c not in table:
            table[c] = len(names)
            names.append(c)
        cid.append(table[c])
        start.append(a)
        end.append(b)
    return names, np.array(cid, np.int64), np.array(start, np.int64), np.array(end, np.int64)


def overlap_map(var_names, peaks):
    """CSR (fptr, fregion) of feature j -> the regions overlapping its
    interval (half-open, start < other end and end > other start), and the
    region names in feature order (repeats dropped, first kept, as the
    reference's interval index set)."""
    seen, regions = set(), []
    for p in peaks:
        r = parse_region(p) if isinstance(p, str) else (str(p[0]), int(p[1]), int(p[2]))
        if r not in seen:
            seen.add(r)
            regions.append(r)
    cnames, fcid, fs, fe = _feature_intervals(var_names)
    m = fs.shape[0]
    ctab = {c: i for i, c in enumerate(cnames)}
    pair_f, pair_r = [], []
    by_chrom: dict = {}
    for k, (c, a, b) in enumerate(regions):
        if c in ctab:
            by_chrom.setdefault(ctab[c], []).append((a, b, k))
    order = np.argsort(fcid, kind="stable")
    bounds = np.searchsorted(fcid[order], np.arange(len(cnames) + 1))
    for c, lst in by_chrom.items():
        a = np.array(lst, dtype=np.int64)
        a = a[np.lexsort((a[:, 0],))]
        rs, re_, rid = a[:, 0], a[:, 1], a[:, 2]
        maxend = np.maximum.accumulate(re_)
        feats = order[bounds[c]:bounds[c + 1]]
        s, e = fs[feats], fe[feats]
        hi = np.searchsorted(rs, e, side="left")        # regions starting before the feature ends
        lo = np.searchsorted(maxend, s, side="right")   # earlier regions all end at or before its start
        cnt = np.maximum(hi - lo, 0)
        if cnt.sum() == 0:
            continue
        f_rep = np.repeat(feats, cnt)
        cand = np.repeat(lo - np.concatenate([[0], np.cumsum(cnt)[:-1]]), cnt) + np.arange(int(cnt.sum()))
        keep = re_[cand] > np.repeat(s, cnt)
        pair_f.append(f_rep[keep])
        pair_r.append(rid[cand[keep]])
    pf = np.concatenate(pair_f) if pair_f else np.zeros(0, np.int64)
    pr = np.concatenate(pair_r) if pair_r else np.zeros(0, np.int64)
    o = np.lexsort((pr, pf))
    pf, pr = pf[o], pr[o]
    fptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(np.bincount(pf, minlength=m), out=fptr[1:])
    names = [f"{c}:{a}-{b}" for c, a, b in regions]
    return fptr, pr.astype(np.int32), names


def aggregate_x(X, var_names, peaks, device=None):
    """``use_x=True``: X (cells x features, CSR: scipy or DeviceCSR) summed
    by regions on the GPU (``sg_csr_aggregate_count`` / ``_run``); the
    overlap map is built on the host from the intervals.  Integer X gives
    uint32 sums, floating X FP64 sums.  Returns (scipy CSR, region names)."""
    from .preprocessing import _device
    dev = _device(device)
    L = _lib.lib()
    fptr, freg, names = overlap_map(var_names, peaks)
    if isinstance(X, DeviceCSR):
        csr = X
        integer = csr.data is None or not torch.is_floating_point(csr.data)
    else:
        Xs = sp.csr_matrix(X)
        Xs.sort_indices()
        integer = np.issubdtype(Xs.dtype, np.integer) or Xs.dtype == bool
        # exact values: integer counts as uint32 bits, anything else as FP64
        data = (np.asarray(Xs.data).astype(np.uint32).view(np.int32) if integer
                else np.asarray(Xs.data, dtype=np.float64))
        csr = DeviceCSR(torch.from_numpy(Xs.indptr.astype(np.int64)).to(dev),
                        torch.from_numpy(Xs.indices.astype(np.int32)).to(dev),
                        torch.from_numpy(np.ascontiguousarray(data)).to(dev), Xs.shape)
    n = csr.shape[0]
    if csr.shape[1] != fptr.shape[0] - 1:
        raise ValueError("var_names and X have different numbers of features")
    dtype = 0 if integer else 1
    if csr.data is None:
        vals = torch.ones(max(csr.nnz, 1), dtype=torch.int32 if integer else torch.float64, device=dev)
    elif integer:
        vals = csr.data.to(torch.int64).clamp_(0, 0xFFFFFFFF).to(torch.int32) if csr.data.dtype != torch.int32 \
            else csr.data
    else:
        vals = csr.data.to(torch.float64)
    sh = torch.cuda.current_stream(dev).cuda_stream
    t_fptr = torch.from_numpy(fptr).to(dev)
    t_freg = torch.from_numpy(freg if freg.size else np.zeros(1, np.int32)).to(dev)
    eoff = torch.empty(n + 1, dtype=torch.int64, device=dev)
    scan = torch.empty(int(L.sg_scan_scratch_bytes(n + 1)), dtype=torch.uint8, device=dev)
    _lib.check(L.sg_csr_aggregate_count(n, csr.indptr.data_ptr(), csr.indices.data_ptr(), t_fptr.data_ptr(),
                                        eoff.data_ptr(), scan.data_ptr(), sh), "sg_csr_aggregate_count")
    E = int(eoff[n].item()) if n else 0
    nb = int(L.sg_csr_aggregate_scratch_bytes(n, E))
    work = torch.empty(nb, dtype=torch.uint8, device=dev)
    cap = max(E, 1)
    out_ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    out_idx = torch.empty(cap, dtype=torch.int32, device=dev)
    out_val = torch.empty(cap, dtype=torch.int32 if integer else torch.float64, device=dev)
    nnz = ctypes.c_int64(0)
    st = _lib.DeviceStatus(dev)
    _lib.check(L.sg_csr_aggregate_run(dtype, n, csr.indptr.data_ptr(), csr.indices.data_ptr(), vals.data_ptr(),
                                      t_fptr.data_ptr(), t_freg.data_ptr(), len(names), eoff.data_ptr(), E,
                                      work.data_ptr(), nb, out_ptr.data_ptr(), out_idx.data_ptr(),
                                      out_val.data_ptr(), cap, ctypes.byref(nnz), st.status_ptr, sh),
               "sg_csr_aggregate_run")
    st.raise_if_error("aggregation by regions")
    k = int(nnz.value)
    data = out_val[:k].cpu().numpy()
    data = data.view(np.uint32) if integer else data
    Y = sp.csr_matrix((data, out_idx[:k].cpu().numpy(), out_ptr.cpu().numpy()), shape=(n, len(names)))
    return Y, names


def make_peak_matrix(adata, *, use_rep=None, inplace: bool = False, file=None, backend="hdf5", peak_file=None,
                     chunk_size: int = 500, use_x: bool = False, min_frag_size: int | None = None,
                     max_frag_size: int | None = None, counting_strategy: str = "paired-insertion",
                     value_type: str = "target", summary_type: str = "sum", device=None):
    """Cell-by-peak count matrix from the fragments (``_basic.py:577-705``).

    Same keywords and outputs: a new AnnData (``X`` uint32 counts, obs
    copied, ``var_names`` "chrom:start-end") or, with ``inplace=True``,
    ``adata.X`` / ``adata.var_names`` replaced.  ``use_x=True`` aggregates
    the existing X by the peaks instead of counting fragments (``_basic.py:
    586,704``).  Backed ``file=`` output is not supported.
    """
    from .preprocessing import _device, _fragment_arrays, read_chrom_sizes
    if counting_strategy not in ("fragment", "insertion", "paired-insertion"):
        raise ValueError("Counting strategy must be one of 'insertion', 'fragment', or 'paired-insertion'")
    if file is not None:
        raise NotImplementedError("backed (file=...) output is not supported; use file=None")
    peaks = _peaks_from(adata, use_rep, peak_file)
    dev = _device(device)
    if use_x:
        X, names = aggregate_x(adata.X, adata.var_names, peaks, dev)
        if inplace:
            if hasattr(adata, "set_n_vars"):
                adata.set_n_vars(X.shape[1])
            adata.X = X
            adata.var_names = names
            return None
        return AnnData(X, obs=dict(getattr(adata, "obs", {}) or {}), obs_names=adata.obs_names, var_names=names)
    cs = read_chrom_sizes(adata)
    paired, indptr, pos, length = _fragment_arrays(adata)
    regions = build_regions(peaks, cs.names, dev)
    t_ptr = torch.from_numpy(indptr).to(dev)
    t_pos = torch.from_numpy(pos).to(dev)
    t_len = torch.from_numpy(np.ascontiguousarray(length).view(np.int32)).to(dev) if paired else None
    res = region_matrix(t_ptr, t_pos, t_len, cs, regions, strategy=counting_strategy if paired else "single",
                        min_frag_size=min_frag_size if paired else None,
                        max_frag_size=max_frag_size if paired else None)
    X = sp.csr_matrix((res.data.cpu().numpy().view(np.uint32), res.indices.cpu().numpy(),
                       res.indptr.cpu().numpy()), shape=res.shape)
    if inplace:
        if hasattr(adata, "set_n_vars"):
            adata.set_n_vars(X.shape[1])
        adata.X = X
        adata.var_names = regions.names
        return None
    return AnnData(X, obs=dict(getattr(adata, "obs", {}) or {}), obs_names=adata.obs_names,
                   var_names=regions.names)


__all__ = ["make_peak_matrix", "build_regions", "region_matrix", "parse_region", "aggregate_x", "overlap_map"]
