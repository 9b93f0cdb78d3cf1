"""Nyström spectral embedding (tl.spectral with sample_size): the
orthogonalisation step on the CPU, and the GPU path against the oracle's
restatement for a given landmark set (GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import nystrom as ony


def _colmatch(A, B, tol):
    """Columns equal up to sign, relative to each column's norm."""
    for j in range(A.shape[1]):
        a, b = A[:, j], B[:, j]
        s = 1.0 if np.dot(a, b) >= 0 else -1.0
        assert np.linalg.norm(a - s * b) <= tol * np.linalg.norm(b), j


def test_orthogonalize_matches_reference_form():
    import torch
    from snapatac2_gb300._nystrom import orthogonalize
    rng = np.random.default_rng(0)
    q = rng.standard_normal((500, 6)) @ np.diag([3.0, 2.0, 1.5, 1.0, 0.5, 0.2])
    ev = np.array([0.9, 0.7, 0.5, 0.3, -0.2, 0.1])
    e_ref, U_ref = ony.orthogonalize(ev, q)
    e, U = orthogonalize(ev, torch.from_numpy(q))
    np.testing.assert_allclose(e, np.real(e_ref), rtol=1e-10, atol=1e-12)
    _colmatch(U.numpy(), np.real(U_ref), 1e-9)


def _data():
    from snapatac2_gb300 import synthetic as syn
    B = syn.binary_csr(3000, 20000, nnz_per_cell=300, n_clusters=4, enriched=4000, seed=11)
    return sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)


@pytest.mark.gpu
@pytest.mark.parametrize("chunk", [20000, 700])
def test_gpu_nystrom_matches_oracle(chunk):
    from snapatac2_gb300._nystrom import spectral_nystrom
    X = _data()
    lm = np.random.default_rng(5).choice(X.shape[0], 800, replace=False)
    k = 12
    v_ref, q_ref = ony.nystrom(X, lm, n_comps=k, chunk_size=chunk)
    e_ref, U_ref = ony.orthogonalize(v_ref, q_ref)
    e, U = spectral_nystrom(X, None, k, 800, landmarks=lm, chunk_size=chunk, precision="fp64")
    np.testing.assert_allclose(e, np.real(e_ref), rtol=1e-6, atol=1e-9)
    _colmatch(U, np.real(U_ref), 1e-5)


@pytest.mark.gpu
def test_gpu_spectral_sample_size_api():
    import snapatac2_gb300 as snap
    X = _data()
    ad = snap.AnnData(X.astype(np.float32))
    snap.tl.spectral(ad, features=None, n_comps=10, sample_size=0.3)
    ev, E = ad.uns["spectral_eigenvalue"], ad.obsm["X_spectral"]
    assert E.shape[0] == X.shape[0] and E.shape[1] == ev.size and np.all(ev > 0)
    snap.tl.spectral(ad, features=None, n_comps=10, sample_size=900, sample_method="degree")
    assert ad.obsm["X_spectral"].shape[0] == X.shape[0]
    with pytest.raises(ValueError):
        snap.tl.spectral(ad, features=None, sample_size=1)


@pytest.mark.gpu
@pytest.mark.parametrize("valued", [False, True])
def test_gpu_light_setup_equals_operator(valued):
    """IDF from column counts and the row norms, without the transpose, give
    the full operator set-up's weights and norms bit for bit."""
    import torch
    from snapatac2_gb300 import _eigen
    from snapatac2_gb300._nystrom import weights_and_norms
    from snapatac2_gb300.tools import csr_to_device
    X = _data()
    if valued:
        X.data = np.random.default_rng(3).integers(1, 4, X.nnz).astype(np.float64)
    csr = csr_to_device(X, torch.device("cuda"))
    w, rinv = weights_and_norms(csr)
    op = _eigen.build_operator(csr)
    assert torch.equal(w, op.w) and torch.equal(rinv, op.rinv)
