"""``snap.pp.make_peak_matrix`` on the GPU: cell-by-region counts.

Drop-in counterpart of ``snapatac2-python/python/snapatac2/preprocessing/_basic.py:577-705``
over the PyO3 ``mk_peak_matrix`` (``snapatac2-python/src/preprocessing.rs:370-430``)
and ``create_peak_matrix`` (``snapatac2-core/src/feature_count/matrix.rs:95-170``).
Region lookup and counting run in ``csrc/region_count.cu`` behind the C ABI
(``sg_region_plan`` / ``sg_region_run`` / ``sg_tile_emit``).
"""
from __future__ import annotations

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


def make_peak_matrix(adata, *, use_rep=None, inplace: bool = False, file=None, backend="hdf5", peak_file=None,
                     chunk_size: int = 500, use_x: bool = False, min_frag_size: int | None = None,
                     max_frag_size: int | None = None, counting_strategy: str = "paired-insertion",
                     value_type: str = "target", summary_type: str = "sum", device=None):
    """Cell-by-peak count matrix from the fragments (``_basic.py:577-705``).

    Same keywords and outputs: a new AnnData (``X`` uint32 counts, obs
    copied, ``var_names`` "chrom:start-end") or, with ``inplace=True``,
    ``adata.X`` / ``adata.var_names`` replaced.  ``use_x`` (aggregating an
    existing X) and backed ``file=`` output are not supported.
    """
    from .preprocessing import _device, _fragment_arrays, read_chrom_sizes
    if counting_strategy not in ("fragment", "insertion", "paired-insertion"):
        raise ValueError("Counting strategy must be one of 'insertion', 'fragment', or 'paired-insertion'")
    if use_x:
        raise NotImplementedError("use_x=True (aggregating X by peaks) is not supported")
    if file is not None:
        raise NotImplementedError("backed (file=...) output is not supported; use file=None")
    peaks = _peaks_from(adata, use_rep, peak_file)
    dev = _device(device)
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


__all__ = ["make_peak_matrix", "build_regions", "region_matrix", "parse_region"]
