"""ORACLE -- test infrastructure only.

Exact kNN graph restating ``snapatac2-core/src/utils/knn.rs:9-31,58-78`` (see
``knn.c``): FP64 squared Euclidean distances, self excluded by index, k
nearest kept, rows sorted by column index, value = sqrt(distance).
"""
from __future__ import annotations

import ctypes

import numpy as np
import scipy.sparse as sp

from ._build import load_lib


def knn_arrays(X: np.ndarray, k: int, q0: int = 0, q1: int | None = None):
    """(nbr int64 [q, k], dist float64 [q, k]) for queries q0..q1-1."""
    lib = load_lib("knn")
    f = lib.oracle_knn
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int64,
                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    X = np.ascontiguousarray(X, dtype=np.float64)
    n, d = X.shape
    q1 = n if q1 is None else q1
    nbr = np.empty((q1 - q0, k), dtype=np.int64)
    dist = np.empty((q1 - q0, k), dtype=np.float64)
    if f(X.ctypes.data, n, d, k, q0, q1, nbr.ctypes.data, dist.ctypes.data) != 0:
        raise ValueError("invalid kNN arguments (need 0 < k <= n - 1)")
    return nbr, dist


def knn_graph(X: np.ndarray, k: int) -> sp.csr_matrix:
    """n x n CSR of Euclidean distances to the k nearest neighbours."""
    n = X.shape[0]
    nbr, dist = knn_arrays(X, k)
    indptr = np.arange(0, n * k + 1, k, dtype=np.int64)
    return sp.csr_matrix((dist.ravel(), nbr.ravel(), indptr), shape=(n, n))
