"""Spectral embedding: oracle pinned to the committed ARPACK fixture (CPU);
GPU operator and eigenpairs against the oracle (GPU).

Tolerances (the path's stated bar): eigenvalues within 1e-5 relative, the
subspaces of the returned (positive) eigenvectors within 1e-4 radians
principal angle, compared up to sign and up to rotations inside clusters of
eigenvalues closer than 1e-3 relative.
Reference: snapatac2-python/src/embedding.rs:24-191,269-326 and
snapatac2-python/python/snapatac2/tools/_embedding.py:223-293; determinism as
in snapatac2-python/tests/test_tools.py:95-123.
"""
import os

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN
from oracle import spectral as osp
from snapatac2_gb300 import synthetic as syn

FIX = np.load(os.path.join(GOLDEN, "spectral.npz"))
EVAL_RTOL = 1e-5
ANGLE_TOL = 1e-4


def fixture_matrix():
    n, m = FIX["shape"]
    return sp.csr_matrix((np.ones(FIX["indices"].shape[0]), FIX["indices"], FIX["indptr"]), shape=(n, m))


def check_eigs(ev, U, ev_ref, U_ref, rtol=EVAL_RTOL, angle=ANGLE_TOL, positive_only=True):
    """Compare top-k-by-magnitude eigenpairs with the reference's."""
    ev, ev_ref = np.asarray(ev), np.asarray(ev_ref)
    assert ev.shape == ev_ref.shape
    # magnitudes, sorted: robust to a sign swap exactly at the |λ| boundary
    a, b = np.sort(np.abs(ev)), np.sort(np.abs(ev_ref))
    assert np.all(np.abs(a - b) <= rtol * b + 1e-12), np.max(np.abs(a - b) / b)
    pos = ev > 0 if positive_only else np.ones(ev.shape, bool)
    pos_ref = ev_ref > 0 if positive_only else np.ones(ev_ref.shape, bool)
    kk = min(pos.sum(), pos_ref.sum())
    assert abs(int(pos.sum()) - int(pos_ref.sum())) <= 1
    o, o_ref = np.argsort(-ev)[:kk], np.argsort(-ev_ref)[:kk]
    ang = osp.eigvec_angles(ev[o], U[:, o], ev_ref[o_ref], U_ref[:, o_ref], rel_gap=1e-3)
    assert ang.max() <= angle, ang
    return ang


# ----------------------------------------------------------------- CPU -----
def test_oracle_reproduces_fixture():
    ev, U = osp.eigen(*osp.operator(fixture_matrix()), 30, 0)
    assert np.allclose(ev, FIX["raw_evals"], rtol=1e-9, atol=1e-12)
    check_eigs(ev, U, FIX["raw_evals"], FIX["raw_evecs"], rtol=1e-9, angle=1e-8)
    evals, evecs = osp.spectral(fixture_matrix(), n_comps=30, random_state=0)
    assert np.allclose(evals, FIX["evals"], rtol=1e-9)


def test_oracle_top_eigenpair_is_degree():
    # (XnXnᵀ - I) 1 = d - 1: the top eigenvalue is exactly 1 with u ∝ sqrt(d-1)
    X = fixture_matrix()
    Xs, dinv = osp.operator(X)
    u = np.sqrt(1.0 / dinv)
    Au = Xs @ (Xs.T @ u) - dinv * u
    assert np.allclose(Au, u, rtol=1e-10)
    assert abs(FIX["raw_evals"][0] - 1.0) < 1e-12


def test_oracle_idf_rules():
    # columns: nnz 2 (== n -> n-1), 1, 0 (-> 1)
    X = sp.csr_matrix(np.array([[1, 1, 0], [1, 0, 0]], dtype=float))
    w = osp.idf(X)
    assert np.allclose(w, [np.log(2 / 1), np.log(2 / 1), np.log(2 / 1)])
    X = sp.csr_matrix(np.array([[1, 0], [0, 1]], dtype=float))  # all counts equal -> ones
    assert np.array_equal(osp.idf(X), [1.0, 1.0])
    X = sp.csr_matrix(np.array([[1, 1, 1], [1, 0, 0], [1, 1, 0]], dtype=float))
    assert np.allclose(osp.idf(X), [np.log(3 / 2), np.log(3 / 2), np.log(3 / 1)])


# ----------------------------------------------------------------- GPU -----
def _gpu_operator(X, features=None, weights=None):
    import torch
    from snapatac2_gb300 import _eigen
    from snapatac2_gb300.tools import csr_to_device
    csr = csr_to_device(X, torch.device("cuda"))
    csr = _eigen.select_columns(csr, features)
    return _eigen.build_operator(csr, weights)


def _apply(op, V, precision):
    import torch
    from snapatac2_gb300 import _lib
    code, tdt = (0, torch.float32) if precision == "mixed" else (1, torch.float64)
    n, B = V.shape
    dev = op.a.device
    Z = torch.from_numpy(np.ascontiguousarray(V)).to(dev, tdt)
    Zs, W = torch.empty_like(Z), torch.empty_like(Z)
    T = torch.empty(op.m, B, dtype=tdt, device=dev)
    L = _lib.load()
    sh = torch.cuda.current_stream().cuda_stream
    w2, a, _ = op.scales(code)
    _lib.check(L.sg_block_finish(code, B, n, Z.data_ptr(), None, 0, 0, None, Zs.data_ptr(), a.data_ptr(), sh), "f")
    op.apply(code, B, Z, Zs, T, W, sh)
    return W.double().cpu().numpy()


@pytest.mark.gpu
@pytest.mark.parametrize("valued", [False, True])
def test_gpu_operator_matches_oracle(valued):
    B = syn.binary_csr(1500, 8000, nnz_per_cell=300, n_clusters=5, enriched=1500, seed=2)
    data = np.ones(B.nnz)
    if valued:
        data = np.random.default_rng(0).integers(1, 6, B.nnz).astype(float)
    X = sp.csr_matrix((data, B.indices, B.indptr), shape=B.shape)
    feats = np.zeros(8000, bool)
    feats[::3] = True
    feats[5000:] = True
    Xs, dinv = osp.operator(X, features=feats)
    op = _gpu_operator(X, feats)
    assert np.allclose(op.dinv.cpu().numpy(), dinv, rtol=1e-12)
    V = np.random.default_rng(1).standard_normal((1500, 8))
    want = Xs @ (Xs.T @ V) - dinv[:, None] * V
    got64 = _apply(op, V, "fp64")
    assert np.max(np.abs(got64 - want)) <= 1e-12 * np.max(np.abs(want))
    got32 = _apply(op, V, "mixed")
    assert np.max(np.abs(got32 - want)) <= 1e-5 * np.max(np.abs(want))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_gpu_spectral_matches_fixture(precision):
    from snapatac2_gb300.tools import spectral_embedding
    ev, U = spectral_embedding(fixture_matrix(), None, 30, 0, precision=precision)
    check_eigs(ev, U, FIX["raw_evals"], FIX["raw_evecs"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision,block", [("mixed", 8), ("fp64", 8), ("mixed", 16), ("mixed", 4), ("mixed", 32)])
def test_gpu_spectral_matches_oracle(precision, block):
    B = syn.binary_csr(4000, 60000, nnz_per_cell=600, n_clusters=8, enriched=6000, seed=13)
    X = sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)
    ev_ref, U_ref = osp.eigen(*osp.operator(X), 30, 0)
    from snapatac2_gb300.tools import spectral_embedding
    ev, U, info = spectral_embedding(X, None, 30, 0, precision=precision, block=block, return_info=True)
    assert info["converged"], info
    check_eigs(ev, U.cpu().numpy(), ev_ref, U_ref)


@pytest.mark.gpu
def test_gpu_spectral_on_tile_counts():
    """Full path on counts >= 2: binning -> select_features -> spectral."""
    import snapatac2_gb300 as snap
    from oracle import binning as ob
    g = syn.make_genome(total=200_000_000, n_chrom=10)
    fm = syn.make_fragments(600, g, enriched_bins=4000, median_frags=3000, seed=17)
    adata = snap.pp.fragments_to_anndata(fm.indptr, fm.pos, fm.length, g)
    snap.pp.add_tile_matrix(adata)
    assert adata.X.data.max() >= 2
    snap.pp.select_features(adata, n_features=50000)
    ip, ix, ct, nc = ob.tile_bin(fm.indptr, fm.pos, fm.length, g)
    Xo = sp.csr_matrix((ct.astype(float), ix, ip), shape=(600, nc))
    feats = np.asarray(adata.var["selected"])
    ev_ref, U_ref = osp.eigen(*osp.operator(Xo, features=feats), 30, 0)
    from snapatac2_gb300.tools import spectral_embedding
    ev, U = spectral_embedding(adata.X, feats, 30, 0)
    check_eigs(ev, U, ev_ref, U_ref)
    snap.tl.spectral(adata)
    e2, E2 = osp.spectral(Xo, features=feats)
    assert adata.obsm["X_spectral"].shape == E2.shape
    assert np.allclose(adata.uns["spectral_eigenvalue"], e2, rtol=EVAL_RTOL)


@pytest.mark.gpu
def test_gpu_spectral_reproducible():
    from snapatac2_gb300.tools import spectral_embedding
    X = fixture_matrix()
    runs = [spectral_embedding(X, None, 30, 0) for _ in range(3)]
    for ev, U in runs[1:]:
        assert np.array_equal(ev, runs[0][0]) and np.array_equal(U, runs[0][1])


@pytest.mark.gpu
def test_gpu_spectral_api_and_edges():
    import snapatac2_gb300 as snap
    X = fixture_matrix()
    ad = snap.AnnData(X.astype(np.uint32))
    with pytest.raises(NameError):
        snap.tl.spectral(ad)
    snap.tl.spectral(ad, features=None)
    assert np.allclose(ad.uns["spectral_eigenvalue"], FIX["evals"], rtol=EVAL_RTOL)
    assert ad.obsm["X_spectral"].shape == FIX["evecs"].shape
    ev, E = snap.tl.spectral(ad, features=None, inplace=False, weighted_by_sd=False)
    assert ev.shape == (30,)
    # n_comps clamp: n_obs - 1
    small = X[:60]
    small = small[np.asarray(small.sum(axis=1)).ravel() > 0]
    ad2 = snap.AnnData(small)
    ev2, _ = snap.tl.spectral(ad2, features=None, n_comps=100, inplace=False, weighted_by_sd=False)
    assert ev2.shape == (min(small.shape[0], small.shape[1]) - 1,)
    ref = osp.eigen(*osp.operator(small), ev2.shape[0], 0)[0]
    assert np.allclose(np.sort(np.abs(ev2)), np.sort(np.abs(ref)), rtol=EVAL_RTOL, atol=1e-12)
    # an empty cell: the reference produces NaN; we refuse it
    Xz = X.tolil()
    Xz[3, :] = 0
    with pytest.raises(ValueError):
        snap.tl.spectral(snap.AnnData(Xz.tocsr()), features=None)


@pytest.mark.gpu
@pytest.mark.parametrize("valued", [False, True])
def test_gpu_transpose_matches_scipy(valued):
    """Deterministic CSR -> CSC: rows ascending within every column, across
    column panels (m > 16384), with empty rows and empty columns."""
    import torch
    from snapatac2_gb300.tools import csr_to_device
    rng = np.random.default_rng(3)
    n, m = 3000, 40000
    X = sp.random(n, m, density=0.002, format="csr", random_state=4)
    X = X.tolil()
    X[5, :] = 0
    X[:, 17000:17100] = 0
    X = X.tocsr()
    X.data = rng.integers(1, 9, X.nnz).astype(float) if valued else np.ones(X.nnz)
    X.sort_indices()
    from snapatac2_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda")
    csr = csr_to_device(X, dev)
    nblk = int(L.sg_transpose_blocks())
    wb = int(L.sg_transpose_work_bytes(n, m, nblk))
    work = torch.empty(wb, dtype=torch.uint8, device=dev)
    colptr = torch.empty(m + 1, dtype=torch.int64, device=dev)
    rowidx = torch.empty(X.nnz, dtype=torch.int32, device=dev)
    cval = torch.empty(X.nnz, dtype=torch.float32, device=dev) if valued else None
    scan = torch.empty(int(L.sg_scan_scratch_bytes(m + 1)), dtype=torch.uint8, device=dev)
    st = _lib.DeviceStatus(dev)
    _lib.check(L.sg_csr_transpose(n, m, csr.indptr.data_ptr(), csr.indices.data_ptr(),
                                  csr.data.data_ptr() if valued else None, nblk, work.data_ptr(), wb,
                                  colptr.data_ptr(), rowidx.data_ptr(), cval.data_ptr() if valued else None,
                                  scan.data_ptr(), st.status_ptr, torch.cuda.current_stream().cuda_stream), "tr")
    st.raise_if_error("transpose")
    C = X.tocsc()
    C.sort_indices()
    assert np.array_equal(colptr.cpu().numpy(), C.indptr)
    assert np.array_equal(rowidx.cpu().numpy(), C.indices)
    if valued:
        assert np.array_equal(cval.cpu().numpy(), C.data.astype(np.float32))


@pytest.mark.gpu
def test_gpu_rejects_duplicate_columns():
    import torch
    from snapatac2_gb300 import _eigen
    from snapatac2_gb300._binning import DeviceCSR
    dev = torch.device("cuda")
    ip = torch.tensor([0, 3, 5], dtype=torch.int64, device=dev)
    ix = torch.tensor([0, 2, 2, 1, 3], dtype=torch.int32, device=dev)  # row 0 repeats column 2
    with pytest.raises(ValueError):
        _eigen.build_operator(DeviceCSR(ip, ix, None, (2, 4)))


@pytest.mark.gpu
def test_gpu_unconverged_solve_warns():
    """A solve stopped before the requested accuracy says so (RuntimeWarning)."""
    from snapatac2_gb300.tools import spectral_embedding
    B = syn.binary_csr(3000, 20000, nnz_per_cell=200, n_clusters=4, enriched=3000, seed=2)
    X = sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)
    with pytest.warns(RuntimeWarning, match="did not reach"):
        spectral_embedding(X, None, 30, 0, precision="mixed", max_restarts=0, tol_vec=1e-15, tol_val=1e-15)
