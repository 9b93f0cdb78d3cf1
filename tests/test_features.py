"""select_features: GPU column counts (sg_col_counts) and the host ranking.

Counts must equal the reference's FP64 chunked sums bit for bit (integer
counts are summed exactly), and the selected mask must be identical to the
oracle's restatement of ``_find_most_accessible_features``, ties included.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import features as of


def count_matrix(n, m, nnz_per_row, seed, heavy=False):
    rng = np.random.default_rng(seed)
    rows = np.repeat(np.arange(n), rng.poisson(nnz_per_row, n))
    # Zipf-like column popularity: many tied counts, a few very frequent columns
    cols = np.minimum((rng.pareto(1.1, rows.size) * 50).astype(np.int64), m - 1)
    vals = rng.integers(1, 5 if not heavy else 60000, rows.size).astype(np.uint32)
    X = sp.csr_matrix((vals, (rows, cols)), shape=(n, m), dtype=np.uint32)
    X.sum_duplicates()
    X.sort_indices()
    return X


def test_host_ranking_matches_oracle():
    from snapatac2_gb300.preprocessing import _find_most_accessible_features
    rng = np.random.default_rng(3)
    for trial in range(20):
        count = rng.integers(0, 40, 5000).astype(np.float64)  # heavy ties and zeros
        for nf in (10, 1000, 4900, 10000):
            a = _find_most_accessible_features(count, 0.005, 0.005, nf)
            b = of.most_accessible(count, 0.005, 0.005, nf)
            assert np.array_equal(a, b)
    allzero = np.zeros(100)
    assert np.array_equal(_find_most_accessible_features(allzero, 0.005, 0.005, 10),
                          of.most_accessible(allzero, 0.005, 0.005, 10))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["u32", "binary", "f32", "heavy"])
def test_gpu_column_counts_exact(kind):
    from snapatac2_gb300.preprocessing import column_counts
    X = count_matrix(3000, 20000, 200, seed=11, heavy=kind == "heavy")
    if kind == "binary":
        X = sp.csr_matrix((np.ones(X.nnz, np.uint32), X.indices, X.indptr), shape=X.shape)
    if kind == "f32":
        X = sp.csr_matrix((X.data.astype(np.float32) * 0.5, X.indices, X.indptr), shape=X.shape)
    got = column_counts(X)
    ref = of.column_counts(X)
    assert got.dtype == np.float64
    assert np.array_equal(got, ref)  # f32: halves of integers, exact in FP64 whatever the order


@pytest.mark.gpu
def test_gpu_column_counts_device_csr_and_errors():
    import torch
    from snapatac2_gb300._binning import DeviceCSR
    from snapatac2_gb300.preprocessing import column_counts
    X = count_matrix(500, 4000, 50, seed=5)
    dev = torch.device("cuda", 0)
    D = DeviceCSR(torch.from_numpy(X.indptr.astype(np.int64)).to(dev), torch.from_numpy(X.indices).to(dev),
                  torch.from_numpy(X.data.view(np.int32)).to(dev), X.shape)
    assert np.array_equal(column_counts(D), of.column_counts(X))
    bad = DeviceCSR(D.indptr, D.indices.clone(), D.data, X.shape)
    bad.indices[7] = 4000
    with pytest.raises(Exception, match="out of range"):
        column_counts(bad)


@pytest.mark.gpu
def test_gpu_select_features_matches_oracle():
    import snapatac2_gb300 as snap
    X = count_matrix(4000, 60000, 300, seed=21)
    ad = snap.AnnData(X)
    snap.pp.select_features(ad, n_features=5000)
    count, mask = of.select_features(X, n_features=5000)
    assert np.array_equal(np.asarray(ad.var["count"]), count)
    assert np.array_equal(np.asarray(ad.var["selected"]), mask)
    m2 = snap.pp.select_features(ad, n_features=5000, inplace=False)
    assert np.array_equal(m2, mask)
