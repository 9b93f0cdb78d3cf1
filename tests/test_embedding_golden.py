"""The oracle's spectral steps and the package's orthogonalisation against
golden outputs of the reference's own Python (CPU): the ``eigen`` and
``nystrom`` functions embedded in snapatac2-python/src/embedding.rs:158-171
and 222-229, ``orthogonalize`` (tools/_embedding.py:397-413), and the
normalisation and degree scaling of ``SpectralMatrixFree.fit``
(tools/_embedding.py:447-458, the Python twin of embedding.rs:133-152,
315-326), run on seeded inputs by ``tests/golden/make_embedding_golden.py``."""
import importlib.util
import os

import numpy as np
import pytest

from oracle import nystrom as ony
from oracle import spectral as osp

_HERE = os.path.dirname(__file__)
GOLDEN = np.load(os.path.join(_HERE, "golden", "embedding.npz"))
_spec = importlib.util.spec_from_file_location("make_embedding_golden",
                                               os.path.join(_HERE, "golden", "make_embedding_golden.py"))
gen = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(gen)


def _cols_match(A, B, tol):
    """Columns equal up to sign, relative to each column's norm."""
    for j in range(B.shape[1]):
        a, b = A[:, j], B[:, j]
        s = 1.0 if np.dot(a, b) >= 0 else -1.0
        assert np.linalg.norm(a - s * b) <= tol * np.linalg.norm(b), j


def test_oracle_eigen_is_the_reference_call():
    Xs, dinv = gen.eigen_inputs()
    ev, U = osp.eigen(Xs, dinv, 8, 0)
    np.testing.assert_allclose(ev, GOLDEN["eigen_evals"], rtol=1e-12)
    _cols_match(U, GOLDEN["eigen_evecs"], 1e-8)


@pytest.mark.parametrize("tag,valued", [("mf", False), ("mfv", True)])
def test_oracle_normalize_and_degree_are_the_reference_python(tag, valued):
    """Rows scaled by 1 / ||x_i ⊙ w|| after the feature weights, the degree
    d = X (Xᵀ 1) - 1 and the rows scaled by d^-1/2: the matrix and 1/d that
    the reference's Python hands to ``_eigen``, for given weights (binary
    matrix and counts); and the eigenvalues of that operator."""
    import scipy.sparse as sp
    X, w = gen.spectral_mf_inputs(valued)
    Xs, dinv = osp.degree_scale(osp.normalize(X, w))
    Xs = sp.csr_matrix(Xs)
    Xs.sort_indices()
    np.testing.assert_allclose(dinv, GOLDEN[f"{tag}_dinv"], rtol=1e-13)
    assert np.array_equal(Xs.indptr, GOLDEN[f"{tag}_xs_indptr"])
    assert np.array_equal(Xs.indices, GOLDEN[f"{tag}_xs_indices"])
    np.testing.assert_allclose(Xs.data, GOLDEN[f"{tag}_xs_data"], rtol=1e-13)
    ev, _ = osp.eigen(Xs, dinv, 8, 0)
    np.testing.assert_allclose(np.sort(ev)[::-1], GOLDEN[f"{tag}_evals"], rtol=1e-10)


def test_oracle_nystrom_chunk_is_the_reference_function():
    seed, sample, evecs, evals = gen.nystrom_inputs()
    q = ony.rescale_chunk(sample @ (seed.T @ evecs), evals)
    np.testing.assert_allclose(q, GOLDEN["nystrom_q"], rtol=1e-12, atol=1e-15)


def test_oracle_orthogonalize_is_the_reference_function():
    evals, q = gen.orthogonalize_inputs()
    e, V = ony.orthogonalize(evals, q)
    np.testing.assert_allclose(np.real(e), GOLDEN["orth_evals"], rtol=1e-12)
    _cols_match(np.real(V), GOLDEN["orth_evecs"], 1e-10)


def test_package_orthogonalize_matches_reference():
    """The package forms σ and V from the k x k Gram matrix of q instead of
    an SVD of q (one n x k x k product on the device)."""
    torch = pytest.importorskip("torch")
    from snapatac2_gb300._nystrom import orthogonalize
    evals, q = gen.orthogonalize_inputs()
    e, V = orthogonalize(evals, torch.from_numpy(q))
    np.testing.assert_allclose(e, GOLDEN["orth_evals"], rtol=1e-10)
    _cols_match(V.numpy(), GOLDEN["orth_evecs"], 1e-8)
