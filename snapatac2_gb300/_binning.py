"""Device-level tile binning through the C ABI (``sg_tile_plan/run/emit``).

Equivalent of the reference's ``create_tile_matrix`` core
(``snapatac2-core/src/feature_count/matrix.rs:26-93``) for fragment data:
builds the output ``GenomeBaseIndex`` (chromosomes minus the excluded ones,
``FragmentData::get_gindex``, ``data_iter.rs:156-173``) and bins every
fragment on the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .genome import ChromSizes, GenomeIndex

STRATEGIES = {"insertion": 0, "fragment": 1, "paired-insertion": 2, "single": 3}


@dataclass
class DeviceCSR:
    """CSR matrix resident on the GPU (int64 indptr, int32 indices, optional values)."""

    indptr: torch.Tensor
    indices: torch.Tensor
    data: torch.Tensor | None  # None = implicit 1.0 (binary pattern)
    shape: tuple[int, int]

    @property
    def nnz(self) -> int:
        return int(self.indices.shape[0])

    def to_scipy(self, dtype=None):
        import scipy.sparse as sp
        ip = self.indptr.cpu().numpy()
        ix = self.indices.cpu().numpy()
        if self.data is None:
            d = np.ones(ix.shape[0], dtype=dtype or np.float64)
        else:
            d = self.data.cpu().numpy()
            if dtype is not None:
                d = d.astype(dtype)
        return sp.csr_matrix((d, ix, ip), shape=self.shape)


@dataclass
class TileLayout:
    """Output tile index of a binning call."""

    index: GenomeIndex          # kept chromosomes, step = bin size
    chrom_end: np.ndarray       # uint64, cumulative lengths over ALL chromosomes
    bin_off: np.ndarray         # uint64, first output tile per chromosome
    excl: np.ndarray            # uint8, 1 = excluded
    n_cols: int


def tile_layout(chrom_sizes: ChromSizes, bin_size: int, exclude_chroms) -> TileLayout:
    names, sizes = chrom_sizes.names, np.asarray(chrom_sizes.sizes, dtype=np.uint64)
    if len(names) == 0:
        raise ValueError("empty chromosome list")
    if np.any(sizes == 0):
        raise ValueError("chromosome lengths must be positive")
    if np.any(sizes >= np.uint64(1 << 32)):
        raise ValueError("chromosomes of 4 Gb or more are not supported")
    if bin_size <= 0 or bin_size >= (1 << 32):
        raise ValueError("bin_size must be in [1, 2^32)")
    # only chromosomes present in the genome are excluded (data_iter.rs:182-189)
    ex = set(exclude_chroms or []) & set(names)
    excl = np.array([1 if n in ex else 0 for n in names], dtype=np.uint8)
    nb = (sizes + np.uint64(bin_size - 1)) // np.uint64(bin_size)
    nb_kept = np.where(excl == 1, np.uint64(0), nb)
    bin_off = np.zeros(len(names), dtype=np.uint64)
    bin_off[1:] = np.cumsum(nb_kept)[:-1]
    n_cols = int(nb_kept.sum())
    if n_cols >= (1 << 31):
        raise ValueError(f"{n_cols} tiles exceed the int32 column index range; use a larger bin_size")
    kept = ChromSizes([(n, int(s)) for n, s, e in zip(names, sizes, excl) if not e])
    index = GenomeIndex(kept, bin_size) if len(kept) else GenomeIndex([("_", 1)], bin_size)
    return TileLayout(index, np.cumsum(sizes, dtype=np.uint64), bin_off, excl, n_cols)


def tile_matrix(indptr: torch.Tensor, pos: torch.Tensor, length: torch.Tensor | None,
                layout: TileLayout, *, bin_size: int, strategy: str,
                min_frag_size: int | None = None, max_frag_size: int | None = None,
                stream: torch.cuda.Stream | None = None) -> DeviceCSR:
    """Bin fragments resident on the GPU.

    indptr: int64 [n+1]; pos: int64/uint64 bits [F] global start index;
    length: int32/uint32 bits [F] (ignored for ``strategy='single'``).
    Returns a DeviceCSR with uint32 counts stored in an int32 tensor.
    """
    L = _lib.lib()
    dev = indptr.device
    n = int(indptr.shape[0] - 1)
    F = int(pos.shape[0])
    if strategy not in STRATEGIES:
        raise ValueError("Counting strategy must be one of 'insertion', 'fragment', or 'paired-insertion'")
    st = STRATEGIES[strategy]
    if length is None:
        length = torch.ones(F, dtype=torch.int32, device=dev)
    if length.shape[0] != F:
        raise ValueError("fragment positions and lengths differ in length")
    for t in (indptr, pos, length):
        if not t.is_contiguous():
            raise ValueError("inputs must be contiguous")
    s = stream or torch.cuda.current_stream(dev)
    sh = s.cuda_stream
    chrom_end = torch.from_numpy(layout.chrom_end.view(np.int64)).to(dev)
    bin_off = torch.from_numpy(layout.bin_off.view(np.int64)).to(dev)
    excl = torch.from_numpy(layout.excl).to(dev)
    nchrom = int(layout.excl.shape[0])
    mn = -1 if min_frag_size is None else int(min_frag_size)
    mx = -1 if max_frag_size is None else int(max_frag_size)
    status = _lib.DeviceStatus(dev)
    key_ptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    scan_scr = torch.empty(int(L.sg_scan_scratch_bytes(n + 1)), dtype=torch.uint8, device=dev)
    genome_args = [chrom_end.data_ptr(), bin_off.data_ptr(), excl.data_ptr(), nchrom, int(bin_size), st, mn, mx]
    _lib.check(L.sg_tile_plan(indptr.data_ptr(), n, F, pos.data_ptr(), length.data_ptr(), *genome_args,
                              key_ptr.data_ptr(), scan_scr.data_ptr(), status.status_ptr, status.bad_ptr, sh),
               "sg_tile_plan")
    status.raise_if_error("tile binning: fragment out of range of its chromosome", "fragment")
    K = int(key_ptr[n].item()) if n > 0 else 0
    nbytes = int(L.sg_tile_scratch_bytes(K))
    scratch = torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)
    out_indptr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    _lib.check(L.sg_tile_run(indptr.data_ptr(), n, F, pos.data_ptr(), length.data_ptr(), *genome_args,
                             key_ptr.data_ptr(), scratch.data_ptr(), nbytes, out_indptr.data_ptr(),
                             scan_scr.data_ptr(), status.status_ptr, status.bad_ptr, sh), "sg_tile_run")
    status.raise_if_error("tile binning")
    nnz = int(out_indptr[n].item()) if n > 0 else 0
    out_idx = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    out_cnt = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    _lib.check(L.sg_tile_emit(n, key_ptr.data_ptr(), scratch.data_ptr(), nbytes, out_indptr.data_ptr(),
                              out_idx.data_ptr(), out_cnt.data_ptr(), nnz, status.status_ptr, sh), "sg_tile_emit")
    status.raise_if_error("tile binning (emit)")
    return DeviceCSR(out_indptr, out_idx[:nnz], out_cnt[:nnz], (n, layout.n_cols))
