"""``snap.tl.spectral`` -- matrix-free cosine spectral embedding on the GPU.

Drop-in counterpart of ``snapatac2-python/python/snapatac2/tools/_embedding.py:129-295``
for ``distance_metric='cosine'`` with the full sample (``sample_size=None``):
same keywords, defaults, ``n_comps`` clamp, ``weighted_by_sd`` post-processing,
and output slots ``uns['spectral_eigenvalue']`` (float64[k']) and
``obsm['X_spectral']`` (float64[n, k']).
"""
from __future__ import annotations

import threading
import warnings
from typing import Literal

import numpy as np
import scipy.sparse as sp
import torch

from . import _eigen
from ._binning import DeviceCSR


# Below this many cells precision='auto' runs the all-FP64 form.
AUTO_FP64_CELLS = 20_000


def _device(device=None) -> torch.device:
    if device is not None:
        return torch.device(device)
    if not torch.cuda.is_available():
        raise RuntimeError("snapatac2_gb300 needs a CUDA GPU (sm_103a); none is available")
    return torch.device("cuda", torch.cuda.current_device())


class _UploadPool:
    """Device buffers reused from call to call for matrices copied in from
    host memory.  A block the allocator has to map afresh pays a first-touch
    cost on its first write (a 1.7 GB copy then took 70-100 ms instead of
    8 ms); a buffer kept here is written at the copy engine's rate.  One
    buffer per (device, dtype), grown on demand, lent for one call at a time
    (a second concurrent call gets its own allocation)."""

    def __init__(self):
        self._free: dict = {}
        self._lock = threading.Lock()

    def take(self, device, dtype, numel: int) -> torch.Tensor:
        with self._lock:
            b = self._free.pop((device, dtype), None)
        if b is None or b.numel() < numel:
            b = torch.empty(max(numel, 1), dtype=dtype, device=device)
        return b

    def give(self, buf: torch.Tensor) -> None:
        key = (buf.device, buf.dtype)
        with self._lock:
            cur = self._free.get(key)
            if cur is None or cur.numel() < buf.numel():
                self._free[key] = buf

    def clear(self) -> None:
        """Drop the pooled buffers (their memory returns to torch's allocator)."""
        with self._lock:
            self._free.clear()

    def pooled_bytes(self) -> int:
        with self._lock:
            return sum(b.numel() * b.element_size() for b in self._free.values())


_UPLOADS = _UploadPool()


def clear_upload_pool() -> None:
    """Release the device buffers kept for host-to-device uploads."""
    _UPLOADS.clear()


def csr_to_device(X, device, borrowed: list | None = None) -> DeviceCSR:
    """The matrix as a DeviceCSR on ``device``.

    Accepts a scipy CSR matrix (values kept only when not all equal to 1) or
    a DeviceCSR whose tensors live on the host (pinned memory gives
    asynchronous copies) or already on the device.  With ``borrowed`` (a
    list), host tensors are copied into pooled device buffers, which are
    appended to the list and must be handed back with ``release_uploads``
    once the call no longer uses the matrix.
    """
    if isinstance(X, DeviceCSR):
        if X.indptr.device == device:
            return X

        def mv(t):
            if t is None:
                return None
            if borrowed is None:
                return t.to(device, non_blocking=True)
            buf = _UPLOADS.take(device, t.dtype, t.numel())
            borrowed.append(buf)
            dst = buf[:t.numel()].view(t.shape)
            dst.copy_(t, non_blocking=True)
            return dst
        return DeviceCSR(mv(X.indptr), mv(X.indices), mv(X.data), X.shape)
    X = sp.csr_matrix(X)
    if not X.has_sorted_indices:
        X = X.copy()
        X.sort_indices()
    data = X.data
    binary = data.size == 0 or bool(np.all(data == 1))
    ip = torch.from_numpy(X.indptr.astype(np.int64, copy=False)).to(device, non_blocking=True)
    ix = torch.from_numpy(X.indices.astype(np.int32, copy=False)).to(device, non_blocking=True)
    val = None
    if not binary:
        if np.any(np.abs(data) >= 2 ** 24) and np.issubdtype(data.dtype, np.integer):
            raise ValueError("count values of 2^24 or more do not fit the float32 value path")
        val = torch.from_numpy(data.astype(np.float32)).to(device, non_blocking=True)
    return DeviceCSR(ip, ix, val, X.shape)


def release_uploads(borrowed: list) -> None:
    """Hand pooled upload buffers back (see ``csr_to_device``)."""
    for b in borrowed:
        _UPLOADS.give(b)
    borrowed.clear()


def spectral_embedding(X, features=None, n_comps: int = 30, random_state: int = 0, feature_weights=None, *,
                       precision: str = "mixed", block: int | None = None, device=None, return_info: bool = False,
                       **solver_kw):
    """(evals, evecs) of the normalised cosine operator, like the PyO3
    ``spectral_embedding`` (``snapatac2-python/src/embedding.rs:24-59``):
    top ``n_comps`` by magnitude, sorted descending; evecs float64 (n, k).

    ``X`` is a scipy CSR matrix or a ``DeviceCSR`` already on the GPU.
    """
    dev = _device(device)
    borrowed: list = []
    try:
        csr = csr_to_device(X, dev, borrowed)
        csr = _eigen.select_columns(csr, features)
        op = _eigen.build_operator(csr, feature_weights)
        res = _eigen.eigsh_lm(op, n_comps, precision=precision, block=block, seed=random_state, **solver_kw)
        del op, csr
    finally:
        release_uploads(borrowed)
    if not res.info["converged"]:
        warnings.warn(f"spectral embedding did not reach the requested accuracy "
                      f"(max residual {max(res.info['residuals']):.2e}, {res.info['restarts']} restarts)",
                      RuntimeWarning, stacklevel=2)
    if return_info:
        return res.evals, res.evecs, res.info
    return res.evals, res.evecs.cpu().numpy()


def spectral(
    adata,
    n_comps: int = 30,
    features: str | np.ndarray | None = "selected",
    random_state: int = 0,
    sample_size: int | float | None = None,
    sample_method: Literal["random", "degree"] = "random",
    chunk_size: int = 20000,
    distance_metric: Literal["jaccard", "cosine"] = "cosine",
    weighted_by_sd: bool = True,
    feature_weights: list[float] | None = None,
    inplace: bool = True,
    *,
    precision: Literal["auto", "mixed", "fp64"] = "auto",
    block: int | None = None,
    device=None,
):
    """Laplacian-eigenmap embedding (``_embedding.py:129-295``), cosine; the full
    sample, or the Nyström extension from ``sample_size`` landmarks.

    Extra keywords: ``precision`` ('mixed': FP32 SpMM and basis, FP64
    Rayleigh-Ritz and a final FP64 correction sweep; 'fp64': all FP64;
    'auto' (default): FP64 below ``AUTO_FP64_CELLS`` cells, where it is cheap
    and where the top eigenvalues reach into a dense bulk whose gaps are
    comparable to the FP32 noise floor, mixed above), ``block`` (Lanczos
    block size; None: chosen by the autotuner per shape class), ``device``.
    """
    np.random.seed(random_state)
    if isinstance(features, str):
        if features in adata.var:
            features = np.asarray(adata.var[features])
        else:
            raise NameError("Please call `select_features` first or explicitly set `features = None`")
    n_comps = min(adata.n_vars - 1, adata.n_obs - 1, n_comps)
    n_sample = adata.shape[0]
    if sample_size is None:
        sample_size = n_sample
    elif isinstance(sample_size, int):
        if sample_size <= 1:
            raise ValueError("when sample_size is an integer, it should be > 1")
        sample_size = min(sample_size, n_sample)
    else:
        if sample_size <= 0.0 or sample_size > 1.0:
            raise ValueError("when sample_size is a float, it should be > 0 and <= 1")
        sample_size = int(sample_size * n_sample)
    if distance_metric != "cosine":
        raise NotImplementedError("only distance_metric='cosine' (matrix-free) is supported")
    if sample_size < n_sample:
        # Nyström (embedding.rs:61-131): landmark solve with random_state 0, and IDF weights: the
        # reference's call (_embedding.py:264) passes neither random_state nor feature_weights
        from ._nystrom import spectral_nystrom
        if feature_weights is not None:
            warnings.warn("feature_weights are not used with sample_size (the reference's Nystrom call "
                          "takes IDF weights); call snapatac2_gb300._nystrom.spectral_nystrom to weight "
                          "the landmarks", stacklevel=2)
        evals, evecs = spectral_nystrom(adata.X, features, n_comps, sample_size,
                                        weighted_by_degree=sample_method != "random", chunk_size=chunk_size,
                                        feature_weights=None, random_state=0, precision=precision,
                                        block=block, device=device)
    else:
        if precision == "auto":
            precision = "fp64" if adata.n_obs < AUTO_FP64_CELLS else "mixed"
        evals, evecs = spectral_embedding(adata.X, features, n_comps, random_state, feature_weights,
                                          precision=precision, block=block, device=device)
    if weighted_by_sd:
        idx = [i for i in range(evals.shape[0]) if evals[i] > 0]
        evals = evals[idx]
        evecs = evecs[:, idx] * np.sqrt(evals)
    if inplace:
        adata.uns["spectral_eigenvalue"] = evals
        adata.obsm["X_spectral"] = evecs
        return None
    return evals, evecs
