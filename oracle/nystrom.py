"""ORACLE (test infrastructure only): the Nyström embedding restated in NumPy/SciPy.

Follows the reference step by step for a given landmark set:

* weights: ``idf`` over all cells (``idf_from_chunks``,
  snapatac2-python/src/embedding.rs:76-84); landmarks normalised with them
  (``normalize``, embedding.rs:98-102);
* landmark solve: ``spectral_mf`` (embedding.rs:133-191) -- degree scaling and
  the same SciPy ``eigsh`` call (oracle ``spectral.eigen``), returning
  d = degree - 1;
* ``nystrom`` (embedding.rs:193-267) including its embedded Python, chunk by
  chunk over all cells;
* ``orthogonalize`` (snapatac2-python/python/snapatac2/tools/_embedding.py:397-413)
  verbatim in NumPy (thin SVD; the reference's full SVD gives the same
  singular values and right vectors).

The reference's landmark draw (rand 0.8 ``StdRng``) is not restated: the
landmarks are an argument.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import spectral as osp


def nystrom(X: sp.csr_matrix, landmarks, n_comps: int = 30, chunk_size: int = 20000, feature_weights=None):
    X = sp.csr_matrix(X, dtype=np.float64)
    X.sort_indices()
    w = np.asarray(feature_weights, dtype=np.float64) if feature_weights is not None else osp.idf(X)
    seed = osp.normalize(sp.csr_matrix(X[np.asarray(landmarks)]), w)
    Xs, dinv = osp.degree_scale(seed)
    v, u = osp.eigen(Xs, dinv, n_comps, 0)
    d = 1.0 / dinv
    evecs = u / np.sqrt(d)[:, None] / v[None, :]
    outs = []
    for r0 in range(0, X.shape[0], chunk_size):
        sample = osp.normalize(sp.csr_matrix(X[r0:r0 + chunk_size]), w)
        outs.append(rescale_chunk(sample @ (seed.T @ evecs), v))
    return v, np.vstack(outs)


def rescale_chunk(q, v):
    """One chunk of the embedded Python of ``nystrom`` (embedding.rs:224-228):
    d = q (Σ q ⊙ λ), d <= 0 -> min positive d (raises when there is none),
    q / sqrt(d).  Returns a new array."""
    q = np.array(q, dtype=np.float64)
    t = q.sum(axis=0) * v
    dd = q @ t.reshape((-1, 1))
    dd[dd <= 0] = np.min(dd[dd > 0])
    np.divide(q, np.sqrt(dd), out=q)
    return q


def orthogonalize(evals, evecs):
    _, sigma, Vt = np.linalg.svd(evecs, full_matrices=False)
    V = Vt.T
    B = np.multiply(V.T, evals.reshape((1, -1))) @ V
    np.multiply(B, sigma.reshape((-1, 1)), out=B)
    np.multiply(B, sigma.reshape((1, -1)), out=B)
    evals_new, evecs_new = np.linalg.eig(B)
    ix = evals_new.argsort()[::-1]
    evals_new = evals_new[ix]
    evecs_new = evecs_new[:, ix]
    np.divide(evecs_new, sigma.reshape((-1, 1)), out=evecs_new)
    return evals_new, evecs @ V @ evecs_new
