"""ORACLE -- test infrastructure only.

FP64 restatement of the reference's matrix-free cosine spectral embedding:

* ``idf``          ``snapatac2-python/src/embedding.rs:269-286``
* ``normalize``    ``snapatac2-python/src/embedding.rs:315-326``
* ``degree``       ``snapatac2-python/src/embedding.rs:139-152`` (``spectral_mf``)
* ``eigen``        ``snapatac2-python/src/embedding.rs:155-188``: the reference
                   calls SciPy's ARPACK ``eigsh`` from embedded Python on the
                   operator v -> X (Xᵀ v) - D v with ``v0 = rand(n)`` after
                   ``numpy.random.seed(seed)``; this module makes the same call
                   on the installed SciPy, so the arithmetic is the reference's.
  ``threaded=True`` evaluates the same operator with an OpenMP C matvec
                   (``gram.c``) for sizes where SciPy's would take minutes.
* ``spectral``     ``snapatac2-python/python/snapatac2/tools/_embedding.py:223-293``
                   (n_comps clamp, ``weighted_by_sd`` filter and scaling).

Pinned: ``eigen`` by golden outputs of the reference's embedded string;
``normalize`` and ``degree_scale`` by golden outputs of the reference's own
Python twin ``SpectralMatrixFree.fit`` (tools/_embedding.py:447-458), both
made by ``tests/golden/make_embedding_golden.py``.  ``idf`` has no reference
test or Python twin: parity unpinned for that formula.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp
from scipy.sparse.linalg import LinearOperator, eigsh


def idf(X: sp.csr_matrix) -> np.ndarray:
    """Per-column nnz count c; all equal -> 1; c==0 -> 1; c==n -> n-1; ln(n/c)."""
    n = X.shape[0]
    c = np.bincount(X.indices, minlength=X.shape[1]).astype(np.float64)
    if np.all(c == c[0]):
        return np.ones(X.shape[1], dtype=np.float64)
    c[c == 0.0] = 1.0
    c[c == float(n)] = float(n) - 1.0
    return np.log(float(n) / c)


def normalize(X: sp.csr_matrix, w: np.ndarray) -> sp.csr_matrix:
    """x_ij <- x_ij w_j / ||(x w)_i||_2 (a zero row gives NaN, as in the reference)."""
    X = X.copy()
    X.data = X.data * w[X.indices]
    sq = np.add.reduceat(X.data * X.data, X.indptr[:-1]) if X.nnz else np.zeros(X.shape[0])
    empty = np.diff(X.indptr) == 0
    sq = np.where(empty, 0.0, sq)
    with np.errstate(divide="ignore", invalid="ignore"):
        norm = np.sqrt(sq)
        X.data = X.data / np.repeat(norm, np.diff(X.indptr))
    return X


def degree_scale(Xn: sp.csr_matrix):
    """colsum = 1ᵀXn; d = Xn colsum; D⁻¹ = 1/(d-1); rows scaled by sqrt(D⁻¹)."""
    col_sum = np.bincount(Xn.indices, weights=Xn.data, minlength=Xn.shape[1])
    deg = Xn @ col_sum
    dinv = 1.0 / (deg - 1.0)
    Xs = sp.diags(np.sqrt(dinv)) @ Xn
    return sp.csr_matrix(Xs), dinv


def _threaded_matvec(X: sp.csr_matrix, D: np.ndarray):
    """f(v) = X (Xᵀ v) - D v by the OpenMP C restatement (``gram.c``)."""
    import ctypes
    from ._build import load_lib
    fn = load_lib("gram").oracle_gram_matvec
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 10
    X = sp.csr_matrix(X, dtype=np.float64)
    X.sort_indices()
    C = sp.csc_matrix(X)
    C.sort_indices()
    ip, ix, dv = (np.ascontiguousarray(X.indptr, np.int64), np.ascontiguousarray(X.indices, np.int32),
                  np.ascontiguousarray(X.data, np.float64))
    cp, ci, cv = (np.ascontiguousarray(C.indptr, np.int64), np.ascontiguousarray(C.indices, np.int32),
                  np.ascontiguousarray(C.data, np.float64))
    Dd = np.ascontiguousarray(D, np.float64)
    n, m = X.shape
    t = np.empty(m)

    def f(v):
        v = np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
        out = np.empty(n)
        if fn(n, m, ip.ctypes.data, ix.ctypes.data, dv.ctypes.data, cp.ctypes.data, ci.ctypes.data,
              cv.ctypes.data, Dd.ctypes.data, v.ctypes.data, t.ctypes.data, out.ctypes.data) != 0:
            raise ValueError("empty operator")
        return out
    return f


def eigen(X: sp.csr_matrix, D: np.ndarray, k: int, seed: int, threaded: bool = False):
    """Same ``eigsh`` call as the reference's embedded ``eigen`` function.

    ``threaded=True`` evaluates the same operator with the OpenMP C matvec
    (``gram.c``) instead of SciPy's single-threaded CSR products: same
    ``eigsh`` arguments and start vector, sums equal to FP64 rounding."""
    np.random.seed(seed)

    def f(v):
        return X @ (v.T @ X).T - D * v

    if threaded:
        f = _threaded_matvec(X, D)  # noqa: F811
    n = X.shape[0]
    A = LinearOperator((n, n), matvec=f, dtype=np.float64)
    evals, evecs = eigsh(A, k=k, v0=np.random.rand(n))
    ix = evals.argsort()[::-1]
    return evals[ix], evecs[:, ix]


def operator(X: sp.csr_matrix, features=None, feature_weights=None):
    """Return (X̂, D⁻¹) with X̂ = diag(sqrt(D⁻¹)) Xn."""
    X = sp.csr_matrix(X, dtype=np.float64)
    if features is not None:
        features = np.asarray(features)
        if features.dtype == bool:
            features = np.flatnonzero(features)
        X = sp.csr_matrix(X[:, features])
    X.sort_indices()
    w = np.asarray(feature_weights, dtype=np.float64) if feature_weights is not None else idf(X)
    Xn = normalize(X, w)
    return degree_scale(Xn)


def spectral(X: sp.csr_matrix, n_vars: int | None = None, features=None, n_comps: int = 30,
             random_state: int = 0, weighted_by_sd: bool = True, feature_weights=None, threaded: bool = False):
    """(evals, X_spectral) as ``snap.tl.spectral(..., distance_metric='cosine')`` produces
    (``threaded``: the eigensolve's matvec by the OpenMP restatement)."""
    n_obs = X.shape[0]
    n_vars = X.shape[1] if n_vars is None else n_vars
    np.random.seed(random_state)
    n_comps = min(n_vars - 1, n_obs - 1, n_comps)
    Xs, dinv = operator(X, features, feature_weights)
    evals, evecs = eigen(Xs, dinv, n_comps, random_state, threaded=threaded)
    if weighted_by_sd:
        idx = [i for i in range(evals.shape[0]) if evals[i] > 0]
        evals = evals[idx]
        evecs = evecs[:, idx] * np.sqrt(evals)
    return evals, evecs


def principal_angles(U: np.ndarray, V: np.ndarray) -> np.ndarray:
    """Principal angles (radians, descending) between the column spaces of U and V."""
    qu, _ = np.linalg.qr(U)
    qv, _ = np.linalg.qr(V)
    # sines of the angles = singular values of the part of V outside span(U):
    # accurate for small angles, unlike arccos of the cosines
    sn = np.linalg.svd(qv - qu @ (qu.T @ qv), compute_uv=False)
    return np.sort(np.arcsin(np.clip(sn, 0.0, 1.0)))[::-1]


def eig_clusters(evals_ref: np.ndarray, rel_gap: float = 1e-3):
    """Index ranges [i, j) of eigenvalues closer than rel_gap (relative)."""
    k = len(evals_ref)
    out, i = [], 0
    while i < k:
        j = i + 1
        while j < k and abs(evals_ref[j] - evals_ref[j - 1]) <= rel_gap * max(abs(evals_ref[j - 1]), 1e-300):
            j += 1
        out.append((i, j))
        i = j
    return out


def eigvec_angles(evals: np.ndarray, U: np.ndarray, evals_ref: np.ndarray, V: np.ndarray,
                  rel_gap: float = 1e-3, next_eval: float | None = None, return_open: bool = False):
    """Largest principal angle of each cluster of eigenvectors.

    Eigenvalues of the reference closer than ``rel_gap`` (relative) form a
    cluster whose subspace is compared as a whole (independent of sign and of
    rotations inside a degenerate cluster).  If ``next_eval`` (the first
    eigenvalue outside the compared set) is within ``rel_gap`` of the last
    one, the last cluster is cut by the set boundary and its subspace is
    ill-conditioned; with ``return_open`` its angle is returned separately as
    (closed_angles, open_angle) instead of being mixed into the list.
    """
    k = min(U.shape[1], V.shape[1])
    cl = eig_clusters(np.asarray(evals_ref)[:k], rel_gap)
    ang = np.array([float(principal_angles(U[:, i:j], V[:, i:j]).max()) for i, j in cl])
    if not return_open:
        return ang
    last = evals_ref[k - 1]
    is_open = next_eval is not None and abs(next_eval - last) <= rel_gap * abs(last)
    if is_open and len(ang) > 0:
        return ang[:-1], float(ang[-1])
    return ang, None
