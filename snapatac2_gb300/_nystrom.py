"""Nyström spectral embedding (``snap.tl.spectral(sample_size=...)``) on the GPU.

Follows ``spectral_embedding_nystrom`` (``snapatac2-python/src/embedding.rs:61-131``)
and ``nystrom`` (``embedding.rs:193-267``), then ``orthogonalize``
(``snapatac2-python/python/snapatac2/tools/_embedding.py:397-413``):

1. IDF weights over all cells (column cell counts, no transpose of the
   whole matrix) and row norms; landmarks drawn uniformly, or with
   probability proportional to 1 / (degree - 1) (``sample_method="degree"``,
   ``compute_degrees`` / ``compute_probs``, ``embedding.rs:328-365``: this
   one needs the full operator set-up, transpose included);
2. the landmark rows, normalised with the global weights, embedded by the
   same matrix-free eigensolver as the full path (``spectral_mf``);
3. every cell extended out of sample with two FP64 SpMM launches
   (W = seedᵀ · (u / sqrt(d) / λ) over the landmarks' CSC, q = X̂ · W over all
   cells), each chunk of ``chunk_size`` rows rescaled by
   sqrt(q · (Σ_chunk q ⊙ λ)) as the reference's per-chunk Python does;
4. ``orthogonalize``: the singular values and right vectors of q from its
   k x k Gram matrix, the k x k eigenproblem on the host, one n x k x k
   product on the device.

The reference draws its landmarks with ``rand::rngs::StdRng::seed_from_u64(2023)``
(rand 0.8, third-party); this module draws them with NumPy's generator
(same distributions: uniform, or successive weighted sampling without
replacement), or takes them from ``landmarks=`` so that results can be
compared for a given landmark set.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _eigen, _lib
from ._binning import DeviceCSR


def select_rows(csr: DeviceCSR, rows: torch.Tensor) -> DeviceCSR:
    """The CSR rows ``rows`` (int64, in that order), on the device
    (``sg_csr_row_ptr`` then ``sg_csr_copy_rows``)."""
    L = _lib.lib()
    dev = csr.indptr.device
    k = int(rows.numel())
    sh = torch.cuda.current_stream(dev).cuda_stream
    if rows.dtype != torch.int64:
        raise ValueError("row indices must be int64")
    if csr.data is not None and csr.data.element_size() != 4:
        raise ValueError("select_rows: 32-bit values expected")
    ptr = torch.empty(k + 1, dtype=torch.int64, device=dev)
    scan = torch.empty(max(int(L.sg_scan_scratch_bytes(k)), 16), dtype=torch.uint8, device=dev)
    _lib.check(L.sg_csr_row_ptr(k, rows.data_ptr() if k else None, csr.indptr.data_ptr(), ptr.data_ptr(),
                                scan.data_ptr(), sh), "sg_csr_row_ptr")
    total = int(ptr[k].item())
    idx = torch.empty(max(total, 1), dtype=torch.int32, device=dev)
    val = None if csr.data is None else torch.empty(max(total, 1), dtype=csr.data.dtype, device=dev)
    _lib.check(L.sg_csr_copy_rows(k, rows.data_ptr() if k else None, csr.indptr.data_ptr(),
                                  csr.indices.data_ptr() if csr.nnz else idx.data_ptr(),
                                  None if val is None else csr.data.data_ptr(), ptr.data_ptr(), idx.data_ptr(),
                                  None if val is None else val.data_ptr(), sh), "sg_csr_copy_rows")
    return DeviceCSR(ptr, idx[:total], None if val is None else val[:total], (k, csr.shape[1]))


def rescale_chunks(q: torch.Tensor, evals: torch.Tensor, chunk_size: int) -> None:
    """Nyström's per-chunk rescaling of q (n x k, FP64) in place
    (``sg_nystrom_rescale``; the embedded Python of ``embedding.rs:222-229``)."""
    L = _lib.lib()
    n, k = q.shape
    st = _lib.DeviceStatus(q.device)
    _lib.check(L.sg_nystrom_rescale(n, k, q.data_ptr(), evals.data_ptr(), int(chunk_size), st.status_ptr,
                                    st.bad_ptr, torch.cuda.current_stream(q.device).cuda_stream),
               "sg_nystrom_rescale")
    try:
        st.raise_if_error("nystrom rescale", "row")
    except _lib.SnapGB300Error as e:
        if e.code == _lib.SG_ERR_NUMERIC:
            raise ValueError(f"the chunk starting at cell {e.bad_index} has no positive degree estimate "
                             "(the reference raises in np.min)") from e
        raise


def _spmm64(rows, ptr, idx, val, inp, out, scale, block, stream):
    L = _lib.load()
    _lib.check(L.sg_spmm(1, block, rows, ptr.data_ptr(), idx.data_ptr(), None if val is None else val.data_ptr(),
                         inp.data_ptr(), out.data_ptr(), scale.data_ptr(), None, None, -1, stream), "sg_spmm (FP64)")


def orthogonalize(evals: np.ndarray, q: torch.Tensor):
    """``orthogonalize`` (``_embedding.py:397-413``): the eigenpairs of
    diag(σ) Vᵀ diag(λ) V diag(σ) from the SVD q = U diag(σ) Vᵀ, mapped back
    through q V diag(1/σ); returns (evals, n x k evecs on the device)."""
    G = (q.T @ q).cpu().numpy()
    lam, V = np.linalg.eigh(G)
    order = np.argsort(lam)[::-1]
    lam, V = lam[order], V[:, order]
    sigma = np.sqrt(np.maximum(lam, 0.0))
    B = np.multiply(V.T, evals.reshape((1, -1))) @ V
    B *= sigma.reshape((-1, 1))
    B *= sigma.reshape((1, -1))
    evals_new, evecs_new = np.linalg.eig(B)
    evals_new, evecs_new = np.real(evals_new), np.real(evecs_new)
    ix = evals_new.argsort()[::-1]
    evals_new, evecs_new = evals_new[ix], evecs_new[:, ix]
    evecs_new = evecs_new / sigma.reshape((-1, 1))
    M = torch.from_numpy(np.ascontiguousarray(V @ evecs_new)).to(q.device)
    return evals_new, q @ M


def weights_and_norms(csr: DeviceCSR, feature_weights=None):
    """(w, rinv) of all cells without the full operator: IDF from the
    columns' cell counts (``sg_col_counts`` of the index pattern, then
    ``sg_idf_from_counts``) unless weights are given, and the row norms
    (``sg_csr_row_norms``).  No transpose of the whole matrix is built."""
    L = _lib.lib()
    dev = csr.indptr.device
    n, m = csr.shape
    sh = torch.cuda.current_stream(dev).cuda_stream
    f64 = dict(dtype=torch.float64, device=dev)
    st = _lib.DeviceStatus(dev)
    if feature_weights is None:
        counts = torch.empty(m, **f64)
        scratch = torch.empty(m, dtype=torch.int64, device=dev)
        _lib.check(L.sg_col_counts(int(csr.nnz), m, csr.indices.data_ptr() if csr.nnz else None, None, None,
                                   counts.data_ptr(), scratch.data_ptr(), st.status_ptr, st.bad_ptr, sh),
                   "sg_col_counts")
        st.raise_if_error("column counts (column index out of range)")
        w = torch.empty(m, **f64)
        mm = torch.empty(2, dtype=torch.int64, device=dev)
        _lib.check(L.sg_idf_from_counts(n, m, counts.data_ptr(), w.data_ptr(), mm.data_ptr(), sh), "sg_idf")
    else:
        _eigen.check_column_indices(csr)       # no column count pass to check them
        w = torch.as_tensor(np.asarray(feature_weights, dtype=np.float64)).to(dev)
        if w.numel() != m:
            raise ValueError(f"feature_weights has {w.numel()} entries, expected {m}")
    rinv = torch.empty(n, **f64)
    _lib.check(L.sg_csr_row_norms(n, csr.indptr.data_ptr(), csr.indices.data_ptr() if csr.nnz else None,
                                  None if csr.data is None else csr.data.data_ptr(), w.data_ptr(), rinv.data_ptr(),
                                  st.status_ptr, st.bad_ptr, sh), "sg_csr_row_norms")
    try:
        st.raise_if_error("row norms", "cell")
    except _lib.SnapGB300Error as e:
        if e.code == _lib.SG_ERR_NUMERIC:
            raise ValueError(f"cell {e.bad_index} has no selected features; the cosine operator is undefined "
                             "(the reference produces NaN)") from e
        raise
    return w, rinv


def spectral_nystrom(X, features=None, n_comps: int = 30, sample_size: int = 1000, *,
                     weighted_by_degree: bool = False, chunk_size: int = 20000, feature_weights=None,
                     landmarks=None, seed: int = 2023, random_state: int = 0, precision: str = "auto",
                     block: int = 8, device=None, return_info: bool = False):
    """(evals, evecs) of the Nyström embedding: evecs float64 (n, k), the
    landmark eigenvalues re-estimated by ``orthogonalize``."""
    from .tools import _device, csr_to_device, release_uploads
    dev = _device(device)
    borrowed: list = []
    try:
        csr = csr_to_device(X, dev, borrowed)
        csr = _eigen.select_columns(csr, features)
        n, m = csr.shape
        if weighted_by_degree and landmarks is None:
            # degrees need the column sums of all normalised rows: the full set-up (with its transpose)
            op = _eigen.build_operator(csr, feature_weights)
            w, rinv = op.w, op.rinv
            inv = op.dinv.cpu().numpy()                       # 1 / (degree - 1)
            del op
            landmarks = np.random.default_rng(seed).choice(n, sample_size, replace=False, p=inv / inv.sum())
        else:
            w, rinv = weights_and_norms(csr, feature_weights)
            if landmarks is None:
                landmarks = np.random.default_rng(seed).choice(n, sample_size, replace=False)
        lm_h = np.asarray(landmarks, dtype=np.int64).ravel()
        if lm_h.size == 0 or lm_h.min() < 0 or lm_h.max() >= n:
            raise ValueError(f"landmarks must be non-empty row indices in [0, {n})")
        lm = torch.from_numpy(lm_h).to(dev)
        seed_csr = select_rows(csr, lm)
        op_s = _eigen.build_operator(seed_csr, w)             # landmarks with the global weights
        if precision == "auto":
            from .tools import AUTO_FP64_CELLS
            precision = "fp64" if op_s.n < AUTO_FP64_CELLS else "mixed"
        # every landmark eigenvector enters the extension and the orthogonalisation
        # (negative ones included), so all are converged to the vector bar
        res = _eigen.eigsh_lm(op_s, n_comps, precision=precision, block=block, seed=random_state,
                              vec_positive_only=False)
        v = np.asarray(res.evals, dtype=np.float64)
        k = v.size
        sh = torch.cuda.current_stream(dev).cuda_stream
        f64 = dict(dtype=torch.float64, device=dev)
        q = torch.empty(n, k, **f64)
        # evecs / sqrt(d) / λ with d = degree - 1 of the landmark graph, then seedᵀ (·) and X̂ (·), 32 columns a launch
        ev = res.evecs * op_s.dinv.sqrt().unsqueeze(1) / torch.from_numpy(v).to(dev).unsqueeze(0)
        for c0 in range(0, k, 32):
            kc = min(32, k - c0)
            blk = 32 if kc > 16 else (16 if kc > 8 else (8 if kc > 4 else 4))
            inp = torch.zeros(op_s.n, blk, **f64)
            inp[:, :kc] = ev[:, c0:c0 + kc] * op_s.rinv.unsqueeze(1)
            W = torch.empty(m, blk, **f64)
            _spmm64(m, op_s.colptr, op_s.rowidx, op_s.cvalues, inp, W, w, blk, sh)
            W *= w.unsqueeze(1)
            Q = torch.empty(n, blk, **f64)
            _spmm64(n, csr.indptr, csr.indices, csr.data, W, Q, rinv, blk, sh)
            q[:, c0:c0 + kc] = Q[:, :kc]
        rescale_chunks(q, torch.from_numpy(v).to(dev), chunk_size)
        evals, evecs = orthogonalize(v, q)
        info = {"landmarks": int(lm.numel()), "landmark_solve": res.info}
        del op_s, csr, seed_csr
    finally:
        release_uploads(borrowed)
    if return_info:
        return evals, evecs, info
    return evals, evecs.cpu().numpy()
