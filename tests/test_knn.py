"""Exact kNN graph: oracle pinned to the committed fixture and to an
independent NumPy brute force (CPU); GPU graph identical to the oracle's (GPU).

Reference: snapatac2-core/src/utils/knn.rs:9-31,58-78 (self excluded by
index, k nearest, sqrt distance, row columns sorted) and
snapatac2-python/python/snapatac2/preprocessing/_knn.py:10-88.  Both sides
compute the FP64 squared distance the same way and break exact ties by the
smaller index, so the graphs must be identical.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import knn as oknn

FIX = np.load(os.path.join(GOLDEN, "knn.npz"))


def numpy_knn(X, k):
    d = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(d, np.inf)
    nbr = np.empty((X.shape[0], k), np.int64)
    for i in range(X.shape[0]):
        o = np.lexsort((np.arange(X.shape[0]), d[i]))[:k]
        nbr[i] = np.sort(o)
    return nbr


# ----------------------------------------------------------------- CPU -----
def test_oracle_reproduces_fixture():
    nbr, dist = oknn.knn_arrays(FIX["X"], int(FIX["k"]))
    assert np.array_equal(nbr, FIX["nbr"])
    assert np.allclose(dist, FIX["dist"], rtol=0, atol=0)


def test_oracle_matches_numpy_bruteforce():
    X = FIX["X"][:120]
    nbr, dist = oknn.knn_arrays(X, 7)
    assert np.array_equal(nbr, numpy_knn(X, 7))
    # duplicate points 3 and 7: each is the other's nearest neighbour at distance 0
    assert 7 in FIX["nbr"][3] and 3 in FIX["nbr"][7]
    row = list(FIX["nbr"][3])
    assert FIX["dist"][3][row.index(7)] == 0.0


def test_oracle_graph_layout():
    G = oknn.knn_graph(FIX["X"][:50], 5)
    assert G.shape == (50, 50) and G.nnz == 250
    assert np.all(np.diff(G.indices.reshape(50, 5), axis=1) > 0)
    assert np.all(G.indices.reshape(50, 5) != np.arange(50)[:, None])


# ----------------------------------------------------------------- GPU -----
def _gpu(X, k, **kw):
    from snapatac2_gb300._knn_api import knn_arrays
    nbr, dist, nfb = knn_arrays(X, k, return_fallbacks=True, **kw)
    return nbr.cpu().numpy(), dist.cpu().numpy(), nfb


@pytest.mark.gpu
def test_gpu_matches_fixture():
    nbr, dist, _ = _gpu(FIX["X"], int(FIX["k"]))
    assert np.array_equal(nbr, FIX["nbr"])
    assert np.array_equal(dist, FIX["dist"])


@pytest.mark.gpu
@pytest.mark.parametrize("n,d,k", [(2, 3, 1), (50, 1, 49), (333, 16, 10), (1000, 30, 50), (5000, 33, 15),
                                   (4097, 64, 100)])
def test_gpu_matches_oracle_shapes(n, d, k):
    rng = np.random.default_rng(n + d)
    X = rng.standard_normal((n, d)) * rng.uniform(0.1, 10, d)
    want_n, want_d = oknn.knn_arrays(X, k)
    nbr, dist, _ = _gpu(X, k)
    assert np.array_equal(nbr, want_n)
    assert np.array_equal(dist, want_d)


@pytest.mark.gpu
def test_gpu_ties_and_duplicates():
    # integer lattice points: many exact distance ties, plus duplicated rows
    rng = np.random.default_rng(3)
    X = rng.integers(0, 4, (2000, 5)).astype(float)
    for k in (5, 30):
        want_n, want_d = oknn.knn_arrays(X, k)
        nbr, dist, nfb = _gpu(X, k)
        assert np.array_equal(nbr, want_n)
        assert np.array_equal(dist, want_d)


@pytest.mark.gpu
def test_gpu_clustered_embedding_large():
    # spectral-like embedding: tight clusters, k = 50 over 20k cells
    rng = np.random.default_rng(7)
    centers = rng.standard_normal((8, 30)) * 0.05
    lab = rng.integers(0, 8, 20000)
    X = centers[lab] + rng.standard_normal((20000, 30)) * 1e-3
    want_n, want_d = oknn.knn_arrays(X, 50)
    nbr, dist, _ = _gpu(X, 50)
    assert np.array_equal(nbr, want_n)
    assert np.array_equal(dist, want_d)


@pytest.mark.gpu
def test_gpu_certificate_fallback_path():
    # many points at nearly equal distance: margin 0 forces the FP64 rescan
    rng = np.random.default_rng(11)
    v = rng.standard_normal((3000, 8))
    X = v / np.linalg.norm(v, axis=1, keepdims=True)
    X[0] = 0.0  # the centre: every other point within 1e-16 relative of distance 1
    want_n, want_d = oknn.knn_arrays(X, 20)
    nbr, dist, nfb = _gpu(X, 20, margin=0)
    assert nfb >= 1
    assert np.array_equal(nbr, want_n) and np.array_equal(dist, want_d)


@pytest.mark.gpu
def test_knn_api():
    import snapatac2_gb300 as snap
    ad = snap.AnnData(n_obs=300, obsm={"X_spectral": FIX["X"]})
    snap.pp.knn(ad, n_neighbors=10)
    G = ad.obsp["distances"]
    assert G.shape == (300, 300) and G.nnz == 3000
    assert np.array_equal(G.indices.reshape(300, 10), FIX["nbr"])
    G2 = snap.pp.knn(FIX["X"], n_neighbors=4, use_dims=5)
    want = oknn.knn_graph(FIX["X"][:, :5], 4)
    assert (G2 != want).nnz == 0
    with pytest.raises(ValueError):
        snap.pp.knn(np.zeros((0, 3)))


@pytest.mark.gpu
@pytest.mark.parametrize("filt", ["tensor", "simt"])
@pytest.mark.parametrize("case", ["single_tile", "partial_tile", "clustered", "lattice_ties", "wide_k", "d17"])
def test_gpu_filters_match_oracle(filt, case, monkeypatch):
    """The tensor-core filter (tcgen05 split-BF16 dot products, d <= 32) and
    the FP32 filter give the oracle's graph; ragged tiles, ties, clusters."""
    if filt == "simt":
        monkeypatch.setenv("SNAPGB300_KNN_FILTER", "simt")
    else:
        monkeypatch.delenv("SNAPGB300_KNN_FILTER", raising=False)
    rng = np.random.default_rng(len(case))
    if case == "single_tile":
        X, k = rng.standard_normal((100, 20)), 10
    elif case == "partial_tile":
        X, k = rng.standard_normal((1000, 30)) * rng.uniform(0.1, 10, 30), 50
    elif case == "clustered":
        c = rng.standard_normal((6, 30)) * 0.05
        X, k = c[rng.integers(0, 6, 6000)] + rng.standard_normal((6000, 30)) * 1e-3, 50
    elif case == "lattice_ties":
        X, k = rng.integers(0, 3, (3000, 32)).astype(float), 20
    elif case == "wide_k":  # k + margin past the tensor path's list: FP32 filter either way
        X, k = rng.standard_normal((3000, 30)), 100
    else:
        X, k = rng.standard_normal((4097, 17)), 60
    want_n, want_d = oknn.knn_arrays(X, k)
    nbr, dist, _ = _gpu(X, k)
    assert np.array_equal(nbr, want_n)
    assert np.array_equal(dist, want_d)
