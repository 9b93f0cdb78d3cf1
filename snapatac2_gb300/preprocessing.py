"""``snap.pp`` functions of the cell-embedding path.

Drop-in counterparts of
``snapatac2-python/python/snapatac2/preprocessing/_basic.py`` (``add_tile_matrix``,
``select_features``) and ``.../preprocessing/_knn.py`` (``knn``), with the same
keywords, defaults and output slots.  The compute runs on the GPU through the
C ABI of ``libsnapgb300.so``; there is no CPU fallback.
"""
from __future__ import annotations

import logging
from typing import Literal

import numpy as np
import scipy.sparse as sp
import torch

from . import _binning
from ._anndata import AnnData
from .genome import ChromSizes, TileNames

FRAGMENT_SINGLE = "fragment_single"   # snapatac2-core/src/feature_count/mod.rs:20
FRAGMENT_PAIRED = "fragment_paired"   # snapatac2-core/src/feature_count/mod.rs:23


def _device(device=None) -> torch.device:
    if device is not None:
        return torch.device(device)
    if not torch.cuda.is_available():
        raise RuntimeError("snapatac2_gb300 needs a CUDA GPU (sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


def read_chrom_sizes(adata) -> ChromSizes:
    """``SnapData::read_chrom_sizes`` (``snapatac2-core/src/feature_count/mod.rs:57-71``)."""
    rs = adata.uns.get("reference_sequences")
    if rs is None:
        raise KeyError("key 'reference_sequences' is not present in the '.uns'")
    names = list(rs["reference_seq_name"])
    sizes = [int(x) for x in rs["reference_seq_length"]]
    return ChromSizes(zip(names, sizes))


def fragments_to_anndata(indptr, pos, length, chrom_sizes, *, obs_names=None, paired: bool = True) -> AnnData:
    """Wrap fragments in the layout ``import_fragments`` produces.

    ``obsm['fragment_paired']`` is an n_cells x genome_size CSR whose column is
    the global 0-based start and whose value is the fragment length
    (``snapatac2-core/src/preprocessing/import.rs:22-30``);
    ``uns['reference_sequences']`` holds the chromosome table.
    """
    cs = chrom_sizes if isinstance(chrom_sizes, ChromSizes) else ChromSizes(chrom_sizes)
    indptr = np.asarray(indptr, dtype=np.int64)
    n = indptr.shape[0] - 1
    m = sp.csr_matrix((np.asarray(length).astype(np.uint32 if paired else np.int32),
                       np.asarray(pos).astype(np.int64), indptr), shape=(n, cs.total_size()))
    uns = {"reference_sequences": {"reference_seq_name": np.array(cs.names, dtype=object),
                                   "reference_seq_length": np.array(cs.sizes, dtype=np.uint64)}}
    key = FRAGMENT_PAIRED if paired else FRAGMENT_SINGLE
    return AnnData(obsm={key: m}, uns=uns, n_obs=n, obs_names=obs_names)


def _fragment_arrays(adata):
    """(paired, indptr, pos, length) of the fragment matrix; single-end first,
    as ``SnapData::get_fragment_iter`` checks it first (``mod.rs:79-91``)."""
    if FRAGMENT_SINGLE in adata.obsm:
        m, paired = adata.obsm[FRAGMENT_SINGLE], False
    elif FRAGMENT_PAIRED in adata.obsm:
        m, paired = adata.obsm[FRAGMENT_PAIRED], True
    else:
        raise KeyError(f"one of the following keys must be present in the '.obsm': "
                       f"'{FRAGMENT_SINGLE}', '{FRAGMENT_PAIRED}'")
    m = sp.csr_matrix(m)
    return paired, m.indptr.astype(np.int64), m.indices.astype(np.int64), m.data


def add_tile_matrix(
    adata,
    *,
    bin_size: int = 500,
    inplace: bool = True,
    chunk_size: int = 500,
    exclude_chroms: list[str] | str | None = ["chrM", "chrY", "M", "Y"],
    min_frag_size: int | None = None,
    max_frag_size: int | None = None,
    counting_strategy: Literal["fragment", "insertion", "paired-insertion"] = "paired-insertion",
    value_type: Literal["target", "total", "fraction"] = "target",
    summary_type: Literal["sum", "mean"] = "sum",
    file=None,
    backend: Literal["hdf5"] = "hdf5",
    n_jobs: int = 8,
    device=None,
):
    """Generate the cell-by-tile count matrix (``_basic.py:454-575``).

    Sets ``adata.X`` (CSR, uint32 counts) and ``adata.var_names``
    (``chrom:start-end`` per tile) in place, or returns a new AnnData when
    ``inplace=False``.  ``chunk_size`` is accepted for compatibility; the GPU
    processes all cells at once.  ``value_type``/``summary_type`` apply to
    base-value matrices only, which this package does not handle.
    """
    if isinstance(exclude_chroms, str):
        exclude_chroms = [exclude_chroms]
    if counting_strategy not in ("fragment", "insertion", "paired-insertion"):
        raise ValueError("Counting strategy must be one of 'insertion', 'fragment', or 'paired-insertion'")
    if value_type not in ("target", "total", "fraction"):
        raise ValueError("Value type must be one of 'target', 'total', or 'fraction'")
    if summary_type not in ("sum", "mean", "count"):
        raise ValueError("Summary type must be one of 'sum', 'mean', or 'count'")
    if file is not None:
        raise NotImplementedError("backed (file=...) output is not supported; use file=None")
    if isinstance(adata, list):
        if not inplace:
            raise ValueError("inplace must be True when adata is a list")
        for a in adata:
            add_tile_matrix(a, bin_size=bin_size, inplace=True, exclude_chroms=exclude_chroms,
                            min_frag_size=min_frag_size, max_frag_size=max_frag_size,
                            counting_strategy=counting_strategy, device=device)
        return None

    dev = _device(device)
    cs = read_chrom_sizes(adata)
    paired, indptr, pos, length = _fragment_arrays(adata)
    layout = _binning.tile_layout(cs, int(bin_size), exclude_chroms)
    strategy = counting_strategy if paired else "single"
    t_ptr = torch.from_numpy(indptr).to(dev)
    t_pos = torch.from_numpy(pos).to(dev)
    t_len = torch.from_numpy(np.ascontiguousarray(length).view(np.int32)).to(dev) if paired else None
    res = _binning.tile_matrix(t_ptr, t_pos, t_len, layout, bin_size=int(bin_size), strategy=strategy,
                               min_frag_size=min_frag_size if paired else None,
                               max_frag_size=max_frag_size if paired else None)
    X = sp.csr_matrix((res.data.cpu().numpy().view(np.uint32), res.indices.cpu().numpy(),
                       res.indptr.cpu().numpy()), shape=res.shape)
    names = TileNames(layout.index)
    if inplace:
        adata.set_n_vars(layout.n_cols) if hasattr(adata, "set_n_vars") else None
        adata.X = X
        adata.var_names = names
        return None
    out = AnnData(X, obs=dict(getattr(adata, "obs", {}) or {}), obs_names=adata.obs_names, var_names=names)
    return out


def _find_most_accessible_features(feature_count, filter_lower_quantile, filter_upper_quantile,
                                   total_features) -> np.ndarray:
    """Rank-trim selection of ``_basic.py:952-967``.

    Features are ordered by count with NumPy's default (introsort) argsort,
    zero-count features are dropped, the lowest/highest quantiles (by rank)
    are trimmed, and the ``total_features`` most accessible are returned.
    """
    order = np.argsort(feature_count)
    nz = np.flatnonzero(feature_count[order] > 0)
    order = order[nz[0]:] if nz.size else order[order.size - 1:]
    n = order.size
    lo = int(filter_lower_quantile * n)
    hi = int(filter_upper_quantile * n)
    order = order[lo:n - hi]
    return order[::-1][:total_features]


def column_counts(X, device=None) -> np.ndarray:
    """FP64 column sums of a cell-by-feature matrix on the GPU (sg_col_counts),
    the ``count`` of ``_basic.py:1053-1056``.  ``X`` is a SciPy sparse matrix
    or a DeviceCSR; integer counts are summed exactly, so the result equals
    the reference's FP64 sums bit for bit."""
    from . import _lib
    from ._binning import DeviceCSR
    L = _lib.lib()
    dev = _device(device)
    if isinstance(X, DeviceCSR):
        n, m = X.shape
        idx = X.indices.to(dev)
        vals = None if X.data is None else X.data.to(dev)
    else:
        X = sp.csr_matrix(X)
        n, m = X.shape
        idx = torch.from_numpy(np.ascontiguousarray(X.indices, dtype=np.int32)).to(dev)
        d = X.data
        integral = d.size == 0 or (d.min() >= 0 and d.max() <= 0xFFFFFFFF and
                                   (d.dtype.kind in "ui" or bool(np.all(d == np.floor(d)))))
        if integral:  # uint32 count bits in an int32 tensor
            vals = torch.from_numpy(np.ascontiguousarray(d.astype(np.uint32)).view(np.int32)).to(dev)
        else:
            vals = torch.from_numpy(np.ascontiguousarray(d, dtype=np.float32)).to(dev)
    if m == 0:
        return np.zeros(0)
    out = torch.empty(m, dtype=torch.float64, device=dev)
    scratch = torch.empty(m, dtype=torch.int64, device=dev)
    st = _lib.DeviceStatus(dev)
    cnt_ptr = val_ptr = None
    if vals is not None:
        if vals.dtype == torch.int32:
            cnt_ptr = vals.data_ptr()
        else:
            vals = vals.to(torch.float32)
            val_ptr = vals.data_ptr()
    sh = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(L.sg_col_counts(int(idx.numel()), m, idx.data_ptr() if idx.numel() else None, cnt_ptr, val_ptr,
                               out.data_ptr(), scratch.data_ptr(), st.status_ptr, st.bad_ptr, sh), "sg_col_counts")
    st.raise_if_error("column counts (column index out of range)")
    return out.cpu().numpy()


def select_features(adata, n_features: int = 500000, filter_lower_quantile: float = 0.005,
                    filter_upper_quantile: float = 0.005, whitelist=None, blacklist=None,
                    max_iter: int = 1, inplace: bool = True, n_jobs: int = 8, verbose: bool = True, *,
                    device=None):
    """Most-accessible-feature selection (``_basic.py:969-1095``).

    The column counts are summed on the GPU (``column_counts``); the ranking
    depends on NumPy's unstable argsort tie order, so it runs on the host as
    in the reference and its mask is shared by every consumer.  Sets
    ``var['count']`` and ``var['selected']`` in place, or returns the mask.
    """
    if isinstance(adata, list):
        res = [select_features(a, n_features, filter_lower_quantile, filter_upper_quantile, whitelist,
                               blacklist, max_iter, inplace, verbose=False, device=device) for a in adata]
        return None if inplace else res
    if whitelist is not None or blacklist is not None:
        raise NotImplementedError("whitelist/blacklist BED filtering is not supported")
    if max_iter > 1:  # the reference iterates while iter < max_iter, from 1 (_basic.py:1067-1068)
        raise NotImplementedError("iterative feature selection (max_iter > 1) is not supported")
    X = adata.X
    count = column_counts(X, device)
    if inplace:
        adata.var["count"] = count
    sel = _find_most_accessible_features(count, filter_lower_quantile, filter_upper_quantile, n_features)
    result = np.zeros(count.shape[0], dtype=bool)
    result[sel] = True
    if verbose:
        logging.info(f"Selected {result.sum()} features.")
    if inplace:
        adata.var["selected"] = result
        return None
    return result
