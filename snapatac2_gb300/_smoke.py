"""One small pass of the path on cuda:0, checked against the oracle.

Used by ``__graft_entry__.smoke()``; the oracle is the checker only.
Stages: tile binning (bit-exact), feature selection, spectral embedding
(eigenvalues within 1e-5 relative, eigenvector subspaces within 1e-4 rad),
exact kNN (identical graph).
"""
from __future__ import annotations

import numpy as np


def run_smoke() -> None:
    import scipy.sparse as sp
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("smoke needs cuda:0")
    torch.cuda.set_device(0)
    from oracle import binning as ob
    from oracle import knn as oknn
    from oracle import spectral as osp
    from . import synthetic as syn
    from . import preprocessing as pp
    from . import tools as tl
    from ._knn_api import knn as knn_fn

    g = syn.make_genome(total=100_000_000, n_chrom=8)
    fm = syn.make_fragments(300, g, enriched_bins=3000, median_frags=3000, seed=1)
    adata = pp.fragments_to_anndata(fm.indptr, fm.pos, fm.length, g)
    pp.add_tile_matrix(adata, bin_size=500)
    want = ob.tile_bin(fm.indptr, fm.pos, fm.length, g, bin_size=500)
    X = adata.X
    if not (np.array_equal(X.indptr, want[0]) and np.array_equal(X.indices, want[1])
            and np.array_equal(X.data, want[2]) and X.shape[1] == want[3]):
        raise AssertionError("smoke: tile matrix differs from the oracle")
    print(f"smoke: tile binning ok ({X.nnz} nnz, {X.shape[1]} tiles)")

    pp.select_features(adata, n_features=20000)
    feats = np.asarray(adata.var["selected"])
    tl.spectral(adata, n_comps=20)
    Xo = sp.csr_matrix((want[2].astype(float), want[1], want[0]), shape=(X.shape[0], want[3]))
    ev_ref, E_ref = osp.spectral(Xo, features=feats, n_comps=20)
    ev = adata.uns["spectral_eigenvalue"]
    if ev.shape != ev_ref.shape or not np.allclose(ev, ev_ref, rtol=1e-5):
        raise AssertionError(f"smoke: eigenvalues differ from the oracle: {ev} vs {ev_ref}")
    ang = osp.eigvec_angles(ev, adata.obsm["X_spectral"], ev_ref, E_ref, rel_gap=1e-3)
    if ang.max() > 1e-4:
        raise AssertionError(f"smoke: eigenvector angle {ang.max():.2e} > 1e-4")
    print(f"smoke: spectral ok ({ev.shape[0]} components, max angle {ang.max():.1e})")

    knn_fn(adata, n_neighbors=15)
    G = adata.obsp["distances"]
    Gr = oknn.knn_graph(adata.obsm["X_spectral"], 15)
    if not (np.array_equal(G.indices, Gr.indices) and np.array_equal(G.data, Gr.data)):
        raise AssertionError("smoke: kNN graph differs from the oracle")
    print("smoke: knn ok")
