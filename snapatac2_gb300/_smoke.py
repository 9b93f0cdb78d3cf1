"""One small pass of the path on cuda:0, checked against the oracle.

Used by ``__graft_entry__.smoke()``; the oracle is the checker only.
"""
from __future__ import annotations

import numpy as np


def run_smoke() -> None:
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("smoke needs cuda:0")
    torch.cuda.set_device(0)
    from oracle import binning as ob
    from . import synthetic as syn
    from . import preprocessing as pp

    g = syn.make_genome(total=100_000_000, n_chrom=8)
    fm = syn.make_fragments(64, g, enriched_bins=5000, median_frags=3000, seed=1)
    adata = pp.fragments_to_anndata(fm.indptr, fm.pos, fm.length, g)
    pp.add_tile_matrix(adata, bin_size=500)
    want = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, bin_size=500)
    X = adata.X
    ok = (np.array_equal(X.indptr, want[0]) and np.array_equal(X.indices, want[1])
          and np.array_equal(X.data, want[2]) and X.shape[1] == want[3])
    if not ok:
        raise AssertionError("smoke: tile matrix differs from the oracle")
    print(f"smoke: tile binning ok ({X.nnz} nnz, {X.shape[1]} tiles)")
