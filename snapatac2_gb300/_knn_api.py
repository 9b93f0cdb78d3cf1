"""``snap.pp.knn`` -- exact Euclidean kNN graph on the GPU.

Drop-in counterpart of ``snapatac2-python/python/snapatac2/preprocessing/_knn.py:10-88``
for ``method='kdtree'`` (exact search): same keywords and defaults; the graph is
an n x n CSR of Euclidean distances (float64) with exactly k entries per row,
columns sorted, stored in ``adata.obsp['distances']``.
"""
from __future__ import annotations

from typing import Literal

import numpy as np
import scipy.sparse as sp
import torch

from . import _lib
from ._anndata import is_anndata


def knn_arrays(X, k: int, *, margin: int = 16, device=None, return_fallbacks: bool = False):
    """(nbr int64 [n, k], dist float64 [n, k]) as torch tensors on the GPU."""
    L = _lib.lib()
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    Xt = torch.as_tensor(np.ascontiguousarray(X, dtype=np.float64)) if not torch.is_tensor(X) else X
    Xt = Xt.to(dev, torch.float64).contiguous()
    n, d = Xt.shape
    if k < 1 or k > n - 1:
        raise ValueError(f"n_neighbors must be in [1, n-1] (got {k} for {n} points)")
    if d > 64:
        raise ValueError("at most 64 dimensions are supported; pass use_dims")
    nbytes = int(L.sg_knn_scratch_bytes(n, d, k, margin))
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    nbr = torch.empty(n, k, dtype=torch.int64, device=dev)
    dist = torch.empty(n, k, dtype=torch.float64, device=dev)
    nfb = torch.zeros(1, dtype=torch.int32, device=dev)
    sh = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(L.sg_knn(Xt.data_ptr(), n, d, k, margin, nbr.data_ptr(), dist.data_ptr(), scratch.data_ptr(),
                        nbytes, nfb.data_ptr(), sh), "sg_knn")
    if return_fallbacks:
        return nbr, dist, int(nfb.item())
    return nbr, dist


def knn(
    adata,
    n_neighbors: int = 50,
    use_dims: int | list[int] | None = None,
    use_rep: str = "X_spectral",
    method: Literal["kdtree", "hora", "pynndescent"] = "kdtree",
    inplace: bool = True,
    random_state: int = 0,
    *,
    device=None,
) -> sp.csr_matrix | None:
    """Neighbourhood graph of observations (``_knn.py:10-88``), exact search."""
    if is_anndata(adata):
        data = adata.obsm[use_rep]
    else:
        inplace = False
        data = adata
    data = np.asarray(data)
    if data.size == 0:
        raise ValueError("matrix is empty")
    if use_dims is not None:
        data = data[:, :use_dims] if isinstance(use_dims, int) else data[:, use_dims]
    if method in ("hora", "pynndescent"):
        raise NotImplementedError(f"method='{method}' (approximate search) is not supported; use 'kdtree'")
    if method != "kdtree":
        raise ValueError("method must be one of 'hora', 'pynndescent', 'kdtree'")
    n = data.shape[0]
    nbr, dist = knn_arrays(data, int(n_neighbors), device=device)
    k = nbr.shape[1]
    indptr = np.arange(0, n * k + 1, k, dtype=np.int64)
    adj = sp.csr_matrix((dist.cpu().numpy().ravel(), nbr.cpu().numpy().ravel(), indptr), shape=(n, n))
    if inplace:
        adata.obsp["distances"] = adj
        return None
    return adj
