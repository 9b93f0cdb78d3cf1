"""ORACLE (test infrastructure only): select_features restated in NumPy.

Follows snapatac2-python/python/snapatac2/preprocessing/_basic.py:
* count: FP64 column sums accumulated over 2000-row chunks (lines 1053-1056);
* ranking: ``_find_most_accessible_features`` (lines 952-967) -- NumPy's
  default argsort of the counts, leading zero-count features dropped, the
  lower/upper quantiles (by rank) trimmed, the top ``total_features`` kept;
* mask: boolean over all features (lines 1078-1079).
"""
import numpy as np
import scipy.sparse as sp


def column_counts(X, chunk: int = 2000) -> np.ndarray:
    """_basic.py:1053-1056: count += X[chunk].sum(axis=0), FP64."""
    X = sp.csr_matrix(X)
    count = np.zeros(X.shape[1])
    for r0 in range(0, X.shape[0], chunk):
        count += np.ravel(X[r0:r0 + chunk].sum(axis=0))
    return count


def most_accessible(feature_count, lower, upper, total_features) -> np.ndarray:
    """_basic.py:952-967, loop for loop."""
    idx = np.argsort(feature_count)
    for i in range(idx.size):
        if feature_count[idx[i]] > 0:
            break
    idx = idx[i:]
    n = idx.size
    n_lower = int(lower * n)
    n_upper = int(upper * n)
    idx = idx[n_lower:n - n_upper]
    return idx[::-1][:total_features]


def select_features(X, n_features=500000, lower=0.005, upper=0.005):
    """(count, mask) as select_features writes them to var."""
    count = column_counts(X)
    mask = np.zeros(X.shape[1], dtype=bool)
    mask[most_accessible(count, lower, upper, n_features)] = True
    return count, mask
