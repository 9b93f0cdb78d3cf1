"""Batched embedding of several independent datasets in one stacked solve.

Each dataset's result must equal its own reference embedding: eigenvalues
within 1e-5 relative and eigenvector subspaces within 1e-4 rad of the
oracle's ARPACK result (as for a single ``snap.tl.spectral`` call).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import spectral as osp
from snapatac2_gb300 import synthetic as syn


def datasets(seed=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(5):
        n = int(rng.integers(600, 2500))
        m = int(rng.integers(4000, 15000))
        B = syn.binary_csr(n, m, nnz_per_cell=float(rng.integers(150, 400)), n_clusters=int(rng.integers(2, 8)),
                           enriched=m // 6, seed=seed * 100 + i)
        out.append(sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("use_graphs", [True, False])
def test_batched_matches_per_dataset_oracle(use_graphs):
    from snapatac2_gb300._batched import spectral_batched
    mats = datasets(1)
    k = 15
    res = spectral_batched(mats, n_comps=k, weighted_by_sd=False, use_graphs=use_graphs)
    for X, (ev, U) in zip(mats, res):
        ev_ref, U_ref = osp.eigen(*osp.operator(X), k, 0)
        a, b = np.sort(np.abs(ev)), np.sort(np.abs(ev_ref))
        assert np.all(np.abs(a - b) <= 1e-5 * b + 1e-12)
        pos, pos_ref = ev > 0, ev_ref > 0
        kk = int(min(pos.sum(), pos_ref.sum()))
        ang = osp.eigvec_angles(ev[:kk], U[:, :kk], ev_ref[:kk], U_ref[:, :kk], rel_gap=1e-3)
        assert ang.max() <= 1e-4, ang


@pytest.mark.gpu
def test_batched_weighted_output_matches_single():
    from snapatac2_gb300._batched import spectral_batched
    mats = datasets(2)[:3]
    res = spectral_batched(mats, n_comps=20)
    for X, (ev, E) in zip(mats, res):
        e2, E2 = osp.spectral(X, n_comps=20)
        assert ev.shape == e2.shape and np.allclose(ev, e2, rtol=1e-5)
        assert E.shape == E2.shape


@pytest.mark.gpu
def test_concurrent_embedding_matches_separate_solves():
    """embed_concurrent (one sg_lanczos per dataset on a pool of streams)
    gives each dataset the eigenpairs of a separate solve."""
    import torch
    from snapatac2_gb300 import _batched, _eigen
    from snapatac2_gb300._binning import DeviceCSR
    from test_spectral import check_eigs
    dev = torch.device("cuda")
    mats = []
    for d, (n, m) in enumerate([(6000, 40000), (2500, 30000), (9000, 50000), (3000, 20000), (4500, 45000)]):
        B = syn.binary_csr(n, m, nnz_per_cell=300, n_clusters=3 + d, enriched=m // 10, seed=50 + d)
        mats.append(DeviceCSR(torch.from_numpy(B.indptr).to(dev), torch.from_numpy(B.indices).to(dev), None,
                              B.shape))
    conc = _batched.embed_concurrent(mats, 20, block=8, streams=3)
    for c, r in zip(mats, conc):
        ref = _eigen.eigsh_lm(_eigen.build_operator(c), 20, block=8)
        assert r.info["converged"]
        check_eigs(r.evals, r.evecs.cpu().numpy(), ref.evals, ref.evecs.cpu().numpy(), rtol=1e-9, angle=1e-6)
