"""Matrix-free cosine spectral operator and its block Krylov-Schur eigensolver.

Replaces the reference's ``spectral_embedding`` / ``spectral_mf`` / ``eigen``
(``snapatac2-python/src/embedding.rs:24-59,133-191``): the reference builds an
owned FP64 CSR, weights it by IDF, L2-normalises the rows, scales them by
``sqrt(1/(d-1))`` and calls SciPy ARPACK ``eigsh(which='LM')`` on
``v -> X̂ (X̂ᵀ v) - D⁻¹ v``.

Here X stays on the GPU as an index-only CSR (plus a CSC built once), the
scalings are folded into two SpMM kernels, and the eigensolver is a
thick-restart block Lanczos (Krylov-Schur) with full two-pass
reorthogonalisation:

* block expansion (GPU): W = A Z; two passes of W -= Q (Qᵀ W); two
  Cholesky-QR passes; the Rayleigh-quotient block and the coupling R are
  written into H (FP64) on the device;
* restart (GPU, FP64): eigendecomposition of the small H (cluster
  Householder reduction, multisection, inverse iteration), Ritz residuals
  ||R y||, convergence test, thick restart Q <- Q Y_keep.

The whole loop is one C call, ``sg_lanczos`` (``csrc/krylov.cu``); the host
reads one small decision record per restart.

``precision='mixed'`` keeps X, the basis and the SpMM in FP32 with FP32
accumulation (cross-CTA sums in FP64); H, R, the Ritz problem and the output
vectors are FP64.  ``precision='fp64'`` runs everything in FP64.
"""
from __future__ import annotations

import ctypes
import math
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib
from ._binning import DeviceCSR

_DT = {"mixed": (0, torch.float32), "fp64": (1, torch.float64)}


@dataclass
class GramOperator:
    """A v = a ⊙ (X (w² ⊙ (Xᵀ (a ⊙ v)))) - dinv ⊙ v on the GPU."""

    n: int
    m: int
    csr: DeviceCSR
    colptr: torch.Tensor
    rowidx: torch.Tensor
    cvalues: torch.Tensor | None
    w: torch.Tensor        # FP64 feature weights
    w2: torch.Tensor       # FP64
    a: torch.Tensor        # FP64 row scale
    dinv: torch.Tensor     # FP64
    w2_32: torch.Tensor
    a32: torch.Tensor
    dinv32: torch.Tensor
    rinv: torch.Tensor | None = None   # FP64 1/||(XW)_i|| (kept for the adjoint)
    row_mask: torch.Tensor | None = None  # uint8 per cell: 0 skips the row (frozen batched datasets)
    col_mask: torch.Tensor | None = None  # uint8 per feature
    timings: dict = field(default_factory=dict)
    variants: dict = field(default_factory=dict)  # (dtype, block) -> (Xᵀ pass, X pass)
    status: object = None  # DeviceStatus of the staged SpMM's bounded waits (created on first use)
    staged_tables: dict = field(default_factory=dict)  # (pass, row bytes) -> segment table (uint8)
    counter: torch.Tensor | None = None  # row counters of the dynamically scheduled SpMM (one per pass)
    order_t: torch.Tensor | None = None  # int32 positions -> CSC rows, longest first (sg_row_order)

    def row_order_t(self, stream: int) -> torch.Tensor:
        """The CSC's rows (features) by descending length, dealt one per
        4-row fetch (``sg_row_order``): the order in which the dynamically
        scheduled Xᵀ pass takes them.  Built once per operator."""
        if self.order_t is None:
            L = _lib.load()
            npos = int(L.sg_row_order_positions(self.m))
            order = torch.empty(max(npos, 1), dtype=torch.int32, device=self.a.device)
            nb = int(L.sg_row_order_scratch_bytes(self.m))
            scratch = torch.empty(nb, dtype=torch.uint8, device=self.a.device)
            _lib.check(L.sg_row_order(self.m, self.colptr.data_ptr(), order.data_ptr(), scratch.data_ptr(), nb,
                                      stream), "sg_row_order")
            self.order_t = order[:npos]
        return self.order_t

    def scales(self, dtype_code: int):
        if dtype_code == 0:
            return self.w2_32, self.a32, self.dinv32
        return self.w2, self.a, self.dinv

    def apply(self, dtype_code: int, block: int, Z, Zs, T, W, stream: int) -> None:
        """W = A Z (Zs = a ⊙ Z precomputed); T is m x block scratch."""
        vt, vx = self.variants.get((dtype_code, block)) or tune_spmm(self, dtype_code, block, Z, Zs, T, W, stream)
        self.spmm_pass(0, vt, dtype_code, block, Zs, T, stream)
        self.spmm_pass(1, vx, dtype_code, block, T, W, stream, Z)

    def spmm_pass(self, which: int, variant: int, dtype_code: int, block: int, inp, out, stream: int,
                  y=None) -> int:
        """One SpMM launch: which = 0 is T = w² ⊙ Xᵀ inp (CSC, rows = features),
        which = 1 is out = a ⊙ X inp - dinv ⊙ y (CSR, rows = cells).  Variants
        below STAGED select the gather kernel (sg_spmm_masked), STAGED + v
        the stage-tiled kernel (sg_spmm_staged), DYN + v the gather kernel
        with dynamic row scheduling (sg_spmm_dyn).  Returns the C status."""
        L = _lib.load()
        w2, a, dinv = self.scales(dtype_code)
        if which == 0:
            rows, cols, ptr, idx = self.m, self.n, self.colptr, self.rowidx
            val = self.cvalues.data_ptr() if self.cvalues is not None else None
            scale, dsh, yp = w2.data_ptr(), None, None
            mask = self.col_mask.data_ptr() if self.col_mask is not None else None
        else:
            rows, cols, ptr, idx = self.n, self.m, self.csr.indptr, self.csr.indices
            val = self.csr.data.data_ptr() if self.csr.data is not None else None
            scale, dsh, yp = a.data_ptr(), dinv.data_ptr(), y.data_ptr()
            mask = self.row_mask.data_ptr() if self.row_mask is not None else None
        if variant >= DYN and dtype_code != 0:
            variant -= DYN  # the dynamic schedule exists for FP32 only: same gathers, static schedule
        if variant >= DYN:
            if self.counter is None:
                self.counter = torch.zeros(2, dtype=torch.int32, device=self.a.device)
            if which == 0 and mask is None and self.m > 0:  # longest features first
                order = self.row_order_t(stream)
                rc = L.sg_spmm_dyn_ordered(dtype_code, block, order.numel(), ptr.data_ptr(), idx.data_ptr(), val,
                                           inp.data_ptr(), out.data_ptr(), scale, dsh, yp, variant - DYN,
                                           order.data_ptr(), self.counter.data_ptr(), stream)
            else:
                rc = L.sg_spmm_dyn(dtype_code, block, rows, ptr.data_ptr(), idx.data_ptr(), val, inp.data_ptr(),
                                   out.data_ptr(), scale, dsh, yp, variant - DYN, mask,
                                   self.counter.data_ptr() + 4 * which, stream)
        elif variant >= STAGED:
            if self.status is None:
                self.status = _lib.DeviceStatus(self.a.device)
            table = self.staged_table(which, dtype_code, block, stream)
            rc = L.sg_spmm_staged(dtype_code, block, rows, cols, ptr.data_ptr(), idx.data_ptr(), val,
                                  table.data_ptr(), inp.data_ptr(), out.data_ptr(), scale, dsh, yp,
                                  variant - STAGED, mask, self.status.status_ptr, stream)
        else:
            rc = L.sg_spmm_masked(dtype_code, block, rows, ptr.data_ptr(), idx.data_ptr(), val, inp.data_ptr(),
                                  out.data_ptr(), scale, dsh, yp, -1, variant, mask, stream)
        _lib.check(rc, "sg_spmm (Xᵀ)" if which == 0 else "sg_spmm (X)")
        return rc


    def staged_table(self, which: int, dtype_code: int, block: int, stream: int) -> torch.Tensor:
        """Segment table of the stage-tiled SpMM for one pass, built once per
        row width (block x element size) and kept with the operator."""
        key = (which, block * (4 if dtype_code == 0 else 8))
        t = self.staged_tables.get(key)
        if t is None:
            L = _lib.load()
            rows, cols = (self.m, self.n) if which == 0 else (self.n, self.m)
            ptr, idx = (self.colptr, self.rowidx) if which == 0 else (self.csr.indptr, self.csr.indices)
            nb = int(L.sg_staged_table_bytes(dtype_code, block, rows, cols))
            # a table larger than half the column indices means segments of a
            # few nonzeros per (row, stage): the staged schedule cannot pay off
            if nb <= 0 or nb > 2 * max(int(idx.numel()), 1):
                raise _lib.SnapGB300Error(_lib.SG_ERR_ARG, "staged SpMM: shape not supported")
            t = torch.empty(nb, dtype=torch.uint8, device=self.a.device)
            _lib.check(L.sg_staged_table(dtype_code, block, rows, cols, ptr.data_ptr(), idx.data_ptr(),
                                         t.data_ptr(), nb, stream), "sg_staged_table")
            self.staged_tables[key] = t
        return t


# Largest Ritz problem (basis + block) the GPU Rayleigh-Ritz holds on one
# thread-block cluster.
RITZ_MAX = 640
# Residual bar (x max|θ|) of the returned vectors: the loosest that kept every
# returned vector within 1e-4 rad of a solution converged to 1e-12 at 100,000
# cells, including the dense cluster of small eigenvalues cut by the k-th /
# (k+1)-th boundary (1e-8 left it at 1.6e-4 rad with block 16; 3e-9: 3e-5).
TOL_VEC = 3e-9

# Residual level (relative to |A|) below which a stalled mixed-precision
# solve is taken to sit at its FP32 noise floor (~ 2^-24 times a few hundred).
FP32_FLOOR = 3e-5

# Variant codes >= STAGED select the stage-tiled SpMM kernel, codes >= DYN the
# gather kernel on a persistent grid with dynamic row chunks (FP32).
STAGED = 100
DYN = 200

_TUNED: dict = {}


def tune_spmm(op: "GramOperator", code: int, block: int, Z, Zs, T, W, stream: int,
              staged: bool = True) -> tuple[int, int]:
    """Pick the fastest SpMM kernel and variant for each pass.

    Candidates: the gather kernel's memory-access variants (same arithmetic,
    same result) and the stage-tiled kernel's variants (same sums in another
    order: rounding-level differences).  Each is timed (CUDA events, one
    warm-up launch + two timed) on this operator's matrices with zero-filled
    block buffers of the caller's shapes as operands.  The choice is cached
    per process for the shape class (dtype, block, n, m, nnz in units of
    2^20, valued, masked) and can be forced with
    SNAPGB300_SPMM_VARIANT=<t>,<x> (codes >= 100 select the staged kernel,
    >= 200 the dynamically scheduled gather kernel).
    """
    import os
    forced = os.environ.get("SNAPGB300_SPMM_VARIANT")
    if forced:
        vt, vx = (int(x) for x in forced.split(","))
        op.variants[(code, block)] = (vt, vx)
        return vt, vx
    key = (code, block, op.n, op.m, op.csr.nnz >> 20, op.csr.data is not None, op.row_mask is not None, staged)
    if key in _TUNED:
        op.variants[(code, block)] = _TUNED[key]
        return _TUNED[key]
    L = _lib.load()
    gather = list(range(int(L.sg_spmm_variants())))
    if code == 1 and block > 8:  # FP64 wide blocks: the deeper unrolls spill
        gather = [v for v in gather if (v & 3) < 2]
    cands = gather + ([STAGED + v for v in range(int(L.sg_spmm_staged_variants()))] if staged else [])
    if code == 0:  # FP32: the same gathers on a persistent grid with dynamic row chunks
        cands += [DYN + v for v in gather]
    # private operands: the caller's blocks hold live solver state
    Z, Zs, T, W = (torch.zeros_like(t) for t in (Z, Zs, T, W))

    def time_pass(which: int, var: int) -> float:
        def launch():
            if which == 0:
                return op.spmm_pass(0, var, code, block, Zs, T, stream)
            return op.spmm_pass(1, var, code, block, T, W, stream, Z)
        try:
            launch()
        except _lib.SnapGB300Error:
            return math.inf  # shape not supported by this variant
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(2):
            launch()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    best = []
    for which in (0, 1):
        times = [time_pass(which, var) for var in cands]
        best.append(cands[int(np.argmin(times))])
    if op.status is not None:
        op.status.raise_if_error("staged SpMM")
    res = (best[0], best[1])
    for which in (0, 1):  # tables of passes that did not pick the staged kernel
        if res[which] < STAGED:
            op.staged_tables.pop((which, block * (4 if code == 0 else 8)), None)
    _TUNED[key] = res
    op.variants[(code, block)] = res
    return res


# When a list, every eigsh_lm call appends (Xᵀ-pass ms, X-pass ms, block
# matvecs, operator, precision code, block): sg_lanczos times each of its
# SpMM launches with CUDA events on its stream, for the benchmark's roofline.
SPMM_EVENTS: list | None = None


def spmm_bytes(op: "GramOperator", dtype_code: int, block: int) -> tuple[int, int]:
    """Algorithmic bytes of the two SpMM launches of one block matvec.

    Xᵀ pass (rows = m, CSC): column pointers 8(m+1), row indices 4 nnz,
    values 4 nnz if present, gathered input Zs read once 4b·n, output T
    written 4b·m, scale 4m.  X pass (rows = n, CSR): 8(n+1) + 4 nnz (+4 nnz),
    T read once 4b·m, W written 4b·n, Z read 4b·n, scale + shift 8n.
    (Element size 8 instead of 4 for the FP64 form.)
    """
    e = 4 if dtype_code == 0 else 8
    nnz = op.csr.nnz
    vb = 4 * nnz if op.csr.data is not None else 0
    n, m, b = op.n, op.m, block
    t_pass = 8 * (m + 1) + 4 * nnz + vb + e * b * n + e * b * m + e * m
    x_pass = 8 * (n + 1) + 4 * nnz + vb + e * b * m + 2 * e * b * n + 2 * e * n
    return t_pass, x_pass


def check_column_indices(csr: DeviceCSR) -> None:
    """Raise ValueError unless every column index lies in [0, m): kernels
    that look a column up in a per-column table (the column map of the
    selection, the weights of the row norms) read it unchecked.  SciPy's CSR
    constructor does not check index bounds by default."""
    if csr.nnz == 0:
        return
    lo, hi = int(csr.indices.min()), int(csr.indices.max())
    if lo < 0 or hi >= csr.shape[1]:
        raise ValueError(f"X must be CSR with column indices in [0, {csr.shape[1]}); found {lo}..{hi}")


def select_columns(csr: DeviceCSR, features: np.ndarray | None) -> DeviceCSR:
    """X[:, features] on the GPU (embedding.rs:36-41)."""
    if features is None:
        return csr
    check_column_indices(csr)
    L = _lib.lib()
    dev = csr.indptr.device
    n, mfull = csr.shape
    feats = np.asarray(features)
    if feats.dtype == bool:
        if feats.shape[0] != mfull:
            raise ValueError("feature mask length differs from the number of columns")
        feats = np.flatnonzero(feats)
    feats = np.unique(feats.astype(np.int64))
    colmap = np.full(mfull, -1, dtype=np.int32)
    colmap[feats] = np.arange(feats.shape[0], dtype=np.int32)
    cm = torch.from_numpy(colmap).to(dev)
    nnz = csr.nnz
    optr = torch.empty(n + 1, dtype=torch.int64, device=dev)
    oidx = torch.empty(max(nnz, 1), dtype=torch.int32, device=dev)
    oval = torch.empty(max(nnz, 1), dtype=torch.float32, device=dev) if csr.data is not None else None
    scan = torch.empty(int(L.sg_scan_scratch_bytes(n + 1)), dtype=torch.uint8, device=dev)
    sh = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(L.sg_csr_select_cols(n, csr.indptr.data_ptr(), csr.indices.data_ptr(),
                                    csr.data.data_ptr() if csr.data is not None else None, cm.data_ptr(),
                                    optr.data_ptr(), oidx.data_ptr(),
                                    oval.data_ptr() if oval is not None else None, scan.data_ptr(), sh),
               "sg_csr_select_cols")
    k = int(optr[n].item())
    return DeviceCSR(optr, oidx[:k], oval[:k] if oval is not None else None, (n, int(feats.shape[0])))


def transpose(csr: DeviceCSR, stream: int | None = None):
    """(colptr, rowidx, cvalues) of X: deterministic CSR -> CSC on the GPU.
    Raises ValueError on unsorted, duplicate or out-of-range column indices."""
    L = _lib.lib()
    dev = csr.indptr.device
    n, m = csr.shape
    sh = torch.cuda.current_stream(dev).cuda_stream if stream is None else stream
    st = _lib.DeviceStatus(dev)
    nblk = int(L.sg_transpose_blocks())
    nblk = max(1, min(nblk, n))
    wbytes = int(L.sg_transpose_work_bytes(n, m, nblk))
    work = torch.empty(wbytes, dtype=torch.uint8, device=dev)
    colptr = torch.empty(m + 1, dtype=torch.int64, device=dev)
    rowidx = torch.empty(max(csr.nnz, 1), dtype=torch.int32, device=dev)
    cval = torch.empty(max(csr.nnz, 1), dtype=torch.float32, device=dev) if csr.data is not None else None
    scan = torch.empty(int(L.sg_scan_scratch_bytes(max(n, m) + 1)), dtype=torch.uint8, device=dev)
    vptr = csr.data.data_ptr() if csr.data is not None else None
    _lib.check(L.sg_csr_transpose(n, m, csr.indptr.data_ptr(), csr.indices.data_ptr(), vptr, nblk,
                                  work.data_ptr(), wbytes, colptr.data_ptr(), rowidx.data_ptr(),
                                  cval.data_ptr() if cval is not None else None, scan.data_ptr(),
                                  st.status_ptr, sh), "sg_csr_transpose")
    del work
    # the set-up kernels that follow index through X: stop here on invalid indices
    try:
        st.raise_if_error("CSR transpose")
    except _lib.SnapGB300Error as e:
        raise ValueError("X must be CSR with sorted, unique, in-range column indices") from e
    return colptr, rowidx[:csr.nnz], cval[:csr.nnz] if cval is not None else None


def build_operator(csr: DeviceCSR, feature_weights=None, csc=None) -> GramOperator:
    """Transpose, IDF weights, row norms and degrees (embedding.rs:42-47,139-152).

    ``csc`` = (colptr, rowidx, cvalues) of the same matrix skips the transpose
    (the batched path assembles it from per-dataset transposes)."""
    L = _lib.lib()
    dev = csr.indptr.device
    n, m = csr.shape
    if n < 2 or m < 1:
        raise ValueError("need at least 2 cells and 1 feature")
    sh = torch.cuda.current_stream(dev).cuda_stream
    st = _lib.DeviceStatus(dev)
    colptr, rowidx, cval = transpose(csr, sh) if csc is None else csc
    vptr = csr.data.data_ptr() if csr.data is not None else None
    f64 = dict(dtype=torch.float64, device=dev)
    f32 = dict(dtype=torch.float32, device=dev)
    w, w2, rinv, colsum = (torch.empty(m, **f64), torch.empty(m, **f64), torch.empty(n, **f64),
                           torch.empty(m, **f64))
    a, dinv = torch.empty(n, **f64), torch.empty(n, **f64)
    w2_32, a32, dinv32 = torch.empty(m, **f32), torch.empty(n, **f32), torch.empty(n, **f32)
    mm = torch.empty(2, dtype=torch.int64, device=dev)
    fw = None
    if isinstance(feature_weights, torch.Tensor):
        fw = feature_weights.to(dev, torch.float64).contiguous()
    elif feature_weights is not None:
        fw = torch.as_tensor(np.asarray(feature_weights, dtype=np.float64)).to(dev)
    if fw is not None:
        if fw.shape[0] != m:
            raise ValueError(f"feature_weights has {fw.shape[0]} entries, expected {m}")
    _lib.check(L.sg_spectral_prepare(n, m, csr.indptr.data_ptr(), csr.indices.data_ptr(), vptr,
                                     colptr.data_ptr(), rowidx.data_ptr(),
                                     cval.data_ptr() if cval is not None else None,
                                     fw.data_ptr() if fw is not None else None, w.data_ptr(), w2.data_ptr(),
                                     w2_32.data_ptr(), rinv.data_ptr(), colsum.data_ptr(), a.data_ptr(),
                                     dinv.data_ptr(), a32.data_ptr(), dinv32.data_ptr(), mm.data_ptr(),
                                     st.status_ptr, st.bad_ptr, sh), "sg_spectral_prepare")
    try:
        st.raise_if_error("spectral set-up", "cell")
    except _lib.SnapGB300Error as e:
        if e.code == _lib.SG_ERR_ARG:
            raise ValueError("X must be CSR with sorted, unique, in-range column indices") from e
        if e.code == _lib.SG_ERR_NUMERIC:
            raise ValueError(f"cell {e.bad_index} has no selected features or shares none with any other "
                             "cell; the cosine operator is undefined (the reference produces NaN)") from e
        raise
    return GramOperator(n, m, csr, colptr, rowidx, cval, w, w2, a, dinv, w2_32, a32, dinv32, rinv)


# Kernels launched by sg_lanczos calls (the library counts its own launches):
# the benchmark adds it to its launch tally.
LANCZOS_LAUNCHES = 0
_COUNT_LOCK = threading.Lock()


def _spmm_choice(op: GramOperator, code: int, block: int, stream: int, staged: bool = True) -> tuple[int, int]:
    """Tuned SpMM kernels of (precision, block) for this operator, tuning
    with scratch blocks of the right shapes on first use.  ``staged=False``
    (the single block matvec of the correction sweep, whose segment table
    sg_lanczos is not given) keeps to the gather kernels."""
    got = op.variants.get((code, block))
    if got is not None and not staged:
        got = tuple(v if v < STAGED or v >= DYN else 1 for v in got)
    if got is None:
        dev, tdt = op.a.device, _DT["mixed" if code == 0 else "fp64"][1]
        z = [torch.empty(op.n, block, dtype=tdt, device=dev) for _ in range(3)]
        t = torch.empty(op.m, block, dtype=tdt, device=dev)
        got = tune_spmm(op, code, block, z[0], z[1], t, z[2], stream, staged=staged)
        del z, t
    for which in (0, 1):  # the stage-tiled kernel needs its segment table
        if STAGED <= got[which] < DYN:
            op.staged_table(which, code, block, stream)
    return got


def eigsh_lm(op: GramOperator, k: int, *, precision: str = "mixed", block: int | None = 8,
             max_basis: int | None = None,
             keep: int | None = None, tol_vec: float = TOL_VEC, tol_val: float = 1e-6, vec_positive_only: bool = True,
             seed: int = 0, max_restarts: int = 200, stream: torch.cuda.Stream | None = None,
             refine: bool = True) -> EigenResult:
    """k eigenpairs of largest magnitude (ARPACK ``which='LM'``) of ``op``,
    by the library's one-call solver ``sg_lanczos`` (thick-restart block
    Lanczos; the Rayleigh-Ritz step, the convergence test and the restart run
    on the GPU in FP64).

    Convergence: every wanted Ritz pair must have ||A y - θ y|| <= tol·max|θ|,
    with ``tol_vec`` for the pairs whose vectors are returned (the positive
    ones when ``vec_positive_only``, which ``weighted_by_sd`` keeps) and
    ``tol_val`` for the rest (whose eigenvalues only decide the LM set).
    ``block=None`` lets ``choose_block`` pick the block size.
    """
    global LANCZOS_LAUNCHES
    if precision not in _DT:
        raise ValueError("precision must be 'mixed' or 'fp64'")
    L = _lib.lib()
    code, tdt = _DT[precision]
    n = op.n
    dev = op.a.device
    if k < 1 or k >= n:
        raise ValueError(f"need 1 <= k < n (k={k}, n={n})")
    chosen = block is None
    if chosen:
        block = choose_block(op, k, precision, stream.cuda_stream if stream is not None else None)
    if block not in (4, 8, 16, 32):
        raise ValueError("block must be 4, 8, 16 or 32")
    if n <= max(4 * (k + block), 2 * block + 64):
        return _dense_small(op, k, code, tdt, block)
    M0, keep0 = _default_basis(k, block, n)
    M = int(max_basis or M0)
    keep = int(keep or keep0)
    M = min(M, (n - block) // block * block)
    keep = min(keep, M - block)
    if keep < k or M % block:
        raise ValueError("basis too small for k")
    if M + block > RITZ_MAX:
        raise ValueError(f"basis + block must be at most {RITZ_MAX} (the GPU Rayleigh-Ritz limit)")
    s = stream or torch.cuda.current_stream(dev)
    sh = s.cuda_stream
    t0 = time.perf_counter()
    vt, vx = _spmm_choice(op, code, block, sh)
    do_refine = bool(refine and precision == "mixed" and k <= 32)
    rvt, rvx = -1, -1  # the sweep's compensated FP32 kernels: library defaults
    nbytes = int(L.sg_lanczos_work_bytes(code, block, k, n, op.m, M, keep))
    if nbytes <= 0:
        raise ValueError("sg_lanczos: unsupported shape")
    work = torch.empty(nbytes, dtype=torch.uint8, device=dev)
    tt = op.staged_tables
    tab_t = tt.get((0, block * (4 if code == 0 else 8)))
    tab_x = tt.get((1, block * (4 if code == 0 else 8)))
    csr = op.csr
    p = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    order_t = op.row_order_t(sh) if op.m > 0 else None
    gop = _lib.GramOp(n, op.m, p(csr.indptr), p(csr.indices), p(csr.data), p(op.colptr), p(op.rowidx),
                      p(op.cvalues), p(op.w2), p(op.a), p(op.dinv), p(op.w2_32), p(op.a32), p(op.dinv32),
                      p(tab_t), p(tab_x), p(order_t), order_t.numel() if order_t is not None else 0)
    opts = _lib.LanczosOpts(M, keep, float(tol_vec), float(tol_val), int(bool(vec_positive_only)), int(max_restarts),
                            int(do_refine), vt, vx, rvt, rvx, int(SPMM_EVENTS is not None))
    info = _lib.LanczosInfo()
    evals = np.empty(k, dtype=np.float64)
    res = np.empty(k, dtype=np.float64)
    U = torch.empty(n, k, dtype=torch.float64, device=dev)
    st = _lib.DeviceStatus(dev)
    rc = L.sg_lanczos(ctypes.byref(gop), code, block, k, int(seed) & 0xFFFFFFFFFFFFFFFF, ctypes.byref(opts),
                      work.data_ptr(), nbytes, evals.ctypes.data, U.data_ptr(), res.ctypes.data, ctypes.byref(info),
                      st.status_ptr, sh)
    if rc == _lib.SG_ERR_NUMERIC:
        raise _lib.SnapGB300Error(rc, "block Lanczos (rank-deficient Krylov block)")
    if rc == _lib.SG_ERR_TIMEOUT:
        raise _lib.SnapGB300Error(rc, "staged SpMM")
    _lib.check(rc, "sg_lanczos")
    del work
    with _COUNT_LOCK:
        LANCZOS_LAUNCHES += int(info.kernel_launches)
    if max_basis is None and info.converged:  # convergence history of the block choice
        _BLOCK_SEEN.setdefault(_shape_class(op, code, k), {})[block] = int(info.block_matvecs) * block
    if SPMM_EVENTS is not None:
        SPMM_EVENTS.append((info.spmm_ms_t, info.spmm_ms_x, int(info.spmm_launches) // 2, op, code, block))
    ph = dict(cycles=info.seconds_cycles, ritz=info.seconds_ritz, restart=info.seconds_restart,
              refine=info.seconds_refine)
    out = dict(block_matvecs=int(info.block_matvecs), vector_matvecs=int(info.block_matvecs) * block,
               restarts=int(info.restarts), basis=int(info.basis), keep=int(info.keep), residuals=res.tolist(),
               converged=bool(info.converged), seconds=time.perf_counter() - t0, precision=precision, block=block,
               next_evals=[float(x) for x in info.next_evals if not math.isnan(x)], phase_seconds=ph,
               kernel_launches=int(info.kernel_launches), spmm_variants=(vt, vx), block_chosen=chosen)
    return EigenResult(evals, U, out)


@dataclass
class EigenResult:
    evals: np.ndarray          # k eigenvalues, descending
    evecs: torch.Tensor        # n x k FP64 on the device
    info: dict


def _default_basis(k: int, block: int, n: int) -> tuple[int, int]:
    """Basis size M and thick-restart size, as the library's default:
    keep ≈ 3.2 k, M ≈ keep + max(18 blocks, 7.5 k), at most the Rayleigh-Ritz
    limit (k = 30: keep 96, M 384 at block 16; measured at 100k cells to need
    6 restarts and 132 block matvecs against 8 and 140 with keep 80 / M 320)."""
    keep = max(k + 2 * block, int(round(3.2 * k)))
    M = keep + max(18 * block, int(round(7.5 * k)))
    M = int(math.ceil(M / block) * block)
    M = min(M, (RITZ_MAX - block) // block * block)
    return M, keep


# Vector matvecs a solve needs at each block size, relative to block 8 (k =
# 30, tol_vec 3e-9, default basis): 100,000 cells 0.83 / 1 / 1.42 / 2.13 and
# 1,000,000 cells - / 1 / 1.45 / - for blocks 4 / 8 / 16 / 32.  The prior of
# the block choice; observed solves of the same shape class replace it.
BLOCK_PRIOR = {4: 0.83, 8: 1.0, 16: 1.43, 32: 2.13}
_BLOCK_CHOICE: dict = {}   # shape class -> (block, predicted seconds per block)
_BLOCK_SEEN: dict = {}     # shape class -> {block: vector matvecs of the last solve}
_RITZ_MS: dict = {}        # basis size -> measured ms of one GPU Rayleigh-Ritz step


def _shape_class(op: GramOperator, code: int, k: int):
    return (code, op.n, op.m, op.csr.nnz >> 20, op.csr.data is not None, k)


def _ritz_ms(M: int, keep: int, stream: int) -> float:
    """Measured time of one GPU Rayleigh-Ritz step at basis M (cached)."""
    if M in _RITZ_MS:
        return _RITZ_MS[M]
    L = _lib.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device="cpu").manual_seed(M)
    A = torch.randn(M, M, generator=g, dtype=torch.float64)
    A = (0.5 * (A + A.T)).to(dev)
    p = min(M, keep + 4)
    nb = int(L.sg_sym_eig_work_bytes(M, p, p))
    work = torch.empty(nb, dtype=torch.uint8, device=dev)
    nw = M if 2 * p >= M else 2 * p
    ev = torch.empty(nw, dtype=torch.float64, device=dev)
    vec = torch.empty(nw, M, dtype=torch.float64, device=dev)
    run = lambda: _lib.check(L.sg_sym_eig(M, A.data_ptr(), M, p, p, ev.data_ptr(), vec.data_ptr(),  # noqa: E731
                                          work.data_ptr(), nb, stream), "sg_sym_eig")
    run()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run()
    e1.record()
    e1.synchronize()
    _RITZ_MS[M] = e0.elapsed_time(e1)
    return _RITZ_MS[M]


def _quick_variants(op: GramOperator, code: int, b: int, Z, Zs, T, W, stream: int) -> tuple[int, int]:
    """Fastest of a few SpMM kernels per pass (one warm and one timed launch
    each): the kernels the full tuner picks most often, so that the block
    choice compares blocks at near-tuned speed without the full search."""
    if code == 0:
        cands = ([DYN + 7, DYN + 5, DYN + 1, 6, 2], [6, 2, DYN + 2, DYN + 6])
    else:
        cands = ([0, 1, 4, 5], [0, 1, 4, 5])
    best = []
    for which, cs in enumerate(cands):
        times = []
        for v in cs:
            def launch():
                if which == 0:
                    op.spmm_pass(0, v, code, b, Zs, T, stream)
                else:
                    op.spmm_pass(1, v, code, b, T, W, stream, Z)
            try:
                launch()
            except _lib.SnapGB300Error:
                times.append(math.inf)
                continue
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            launch()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        best.append(cs[int(np.argmin(times))])
    return best[0], best[1]


def _block_step_ms(op: GramOperator, code: int, b: int, ncols: int, ld: int, stream: int) -> float:
    """CUDA-event time of one block step at block b: the operator with
    quick-tuned SpMM kernels (``_quick_variants``), two Gram-Schmidt passes
    against ncols basis vectors, two Cholesky-QR passes (scratch operands)."""
    L = _lib.load()
    dev = op.a.device
    tdt = torch.float32 if code == 0 else torch.float64
    n = op.n
    Q = torch.empty(n, ld, dtype=tdt, device=dev)
    Z, Zs, W = (torch.empty(n, b, dtype=tdt, device=dev) for _ in range(3))
    T = torch.empty(op.m, b, dtype=tdt, device=dev)
    nparts = int(L.sg_proj_parts())
    f64 = dict(dtype=torch.float64, device=dev)
    part, C = torch.empty(nparts * ld * b, **f64), torch.empty(ld * b, **f64)
    G, R, Ri = (torch.empty(b * b, **f64) for _ in range(3))
    st = _lib.DeviceStatus(dev)
    for t in (Q, Z, Zs, W):
        _lib.check(L.sg_fill_random(code, t.numel(), 7, t.data_ptr(), stream), "fill")
    vt, vx = _quick_variants(op, code, b, Z, Zs, T, W, stream)

    def step():
        op.spmm_pass(0, vt, code, b, Zs, T, stream)
        op.spmm_pass(1, vx, code, b, T, W, stream, Z)
        for _ in range(2):
            L.sg_block_proj(code, b, n, Q.data_ptr(), ld, ncols, W.data_ptr(), part.data_ptr(), nparts,
                            C.data_ptr(), stream)
            L.sg_block_update(code, b, n, Q.data_ptr(), ld, ncols, C.data_ptr(), W.data_ptr(), stream)
        for _ in range(2):
            L.sg_block_cholqr(code, b, n, W.data_ptr(), part.data_ptr(), nparts, G.data_ptr(), R.data_ptr(),
                              Ri.data_ptr(), st.status_ptr, stream)
    step()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    step()
    e1.record()
    e1.synchronize()
    return e0.elapsed_time(e1)


def choose_block(op: GramOperator, k: int, precision: str = "mixed", stream: int | None = None,
                 candidates=(4, 8, 16, 32)) -> int:
    """Lanczos block size for this operator, chosen once per shape class
    (precision, n, m, nnz, valued, k) and process.

    For each candidate b the predicted solve time is
      V(b)/b x (one block step, measured) + V(b)/(M_b - keep_b) x (one GPU
      Rayleigh-Ritz step at basis M_b, measured),
    with V(b) the vector matvecs the solve needs: the observed count of an
    earlier solve of this shape class at block b, else BLOCK_PRIOR scaled by
    the observed counts at other blocks.  Block steps are timed on scratch
    operands with quick-tuned SpMM kernels (the full kernel search runs
    afterwards for the chosen block only: searching every block costs
    seconds at 1M cells).
    """
    code = _DT[precision][0]
    key = _shape_class(op, code, k)
    if key in _BLOCK_CHOICE:
        return _BLOCK_CHOICE[key][0]
    n = op.n
    dev = op.a.device
    sh = stream if stream is not None else torch.cuda.current_stream(dev).cuda_stream
    seen = _BLOCK_SEEN.get(key, {})
    scale = np.mean([v / BLOCK_PRIOR[b] for b, v in seen.items()]) if seen else 1.0
    best, pred = 8, {}
    for b in candidates:
        if n <= max(4 * (k + b), 2 * b + 64):
            continue
        M, keep = _default_basis(k, b, n)
        M = min(M, (n - b) // b * b)
        keep = min(keep, M - b)
        if keep < k or M + b > RITZ_MAX:
            continue
        V = seen.get(b, BLOCK_PRIOR[b] * scale)
        t_step = _block_step_ms(op, code, b, (keep + M) // 2, M + b, sh)
        t_rr = _ritz_ms(M, keep, sh)
        pred[b] = V / b * t_step + V / (M - keep) * t_rr
    if pred:
        best = min(pred, key=pred.get)
    _BLOCK_CHOICE[key] = (best, pred)
    return best


def eigsh_lm_host_ritz(op: GramOperator, k: int, *, precision: str = "mixed", block: int = 8,
                       max_basis: int | None = None, keep: int | None = None, tol_vec: float = TOL_VEC,
                       tol_val: float = 1e-6, vec_positive_only: bool = True, seed: int = 0, max_restarts: int = 200,
                       stream: torch.cuda.Stream | None = None, refine: bool = True) -> EigenResult:
    """The same solver driven step by step from Python with the Ritz problem
    solved on the host (LAPACK): the driver before ``sg_lanczos``, kept to
    check the one-call solver against it and to time the two Rayleigh-Ritz
    placements side by side.

    Convergence: every wanted Ritz pair must have ||A y - θ y|| <= tol·max|θ|,
    with ``tol_vec`` for the pairs whose vectors are returned (the positive
    ones when ``vec_positive_only``, which ``weighted_by_sd`` keeps) and
    ``tol_val`` for the rest (whose eigenvalues only decide the LM set).
    """
    if precision not in _DT:
        raise ValueError("precision must be 'mixed' or 'fp64'")
    if block not in (4, 8, 16, 32):
        raise ValueError("block must be 4, 8, 16 or 32")
    L = _lib.lib()
    code, tdt = _DT[precision]
    n = op.n
    dev = op.a.device
    if k < 1 or k >= n:
        raise ValueError(f"need 1 <= k < n (k={k}, n={n})")
    if n <= max(4 * (k + block), 2 * block + 64):
        return _dense_small(op, k, code, tdt, block)
    M0, keep0 = _default_basis(k, block, n)
    M = int(max_basis or M0)
    keep = int(keep or keep0)
    M = min(M, (n - block) // block * block)
    keep = min(keep, M - block)
    if keep < k or M % block:
        raise ValueError("basis too small for k")
    s = stream or torch.cuda.current_stream(dev)
    sh = s.cuda_stream
    ld = M + block
    kw = dict(dtype=tdt, device=dev)
    Q = torch.empty(n, ld, **kw)
    Q2 = torch.empty(n, ld, **kw)
    Z, Zs, W = torch.empty(n, block, **kw), torch.empty(n, block, **kw), torch.empty(n, block, **kw)
    T = torch.empty(op.m, block, **kw)
    nparts = int(L.sg_proj_parts())
    f64 = dict(dtype=torch.float64, device=dev)
    part = torch.empty(nparts * ld * block, **f64)
    C1, C2 = torch.empty(ld * block, **f64), torch.empty(ld * block, **f64)
    G = torch.empty(block * block, **f64)
    R1, R2, Rinv, Rout = (torch.empty(block * block, **f64) for _ in range(4))
    H = torch.zeros(ld, ld, **f64)
    st = _lib.DeviceStatus(dev)
    w2, a, dinv = op.scales(code)
    t0 = time.perf_counter()

    def cholqr2():
        _lib.check(L.sg_block_cholqr(code, block, n, W.data_ptr(), part.data_ptr(), nparts, G.data_ptr(),
                                     R1.data_ptr(), Rinv.data_ptr(), st.status_ptr, sh), "cholqr")
        _lib.check(L.sg_block_cholqr(code, block, n, W.data_ptr(), part.data_ptr(), nparts, G.data_ptr(),
                                     R2.data_ptr(), Rinv.data_ptr(), st.status_ptr, sh), "cholqr")

    # start block: deterministic uniform noise, orthonormalised
    _lib.check(L.sg_fill_random(code, n * block, int(seed) & 0xFFFFFFFFFFFFFFFF, W.data_ptr(), sh), "fill")
    cholqr2()
    _lib.check(L.sg_block_finish(code, block, n, W.data_ptr(), Q.data_ptr(), ld, 0, Z.data_ptr(),
                                 Zs.data_ptr(), a.data_ptr(), sh), "finish")
    m = 0
    n_mv = 0
    restarts = 0
    hist = []
    ph = dict(cycles=0.0, ritz=0.0, restart=0.0, refine=0.0)
    while True:
        tc = time.perf_counter()
        while m + block <= M:
            op.apply(code, block, Z, Zs, T, W, sh)
            n_mv += 1
            ncols = m + block
            for C in (C1, C2):
                _lib.check(L.sg_block_proj(code, block, n, Q.data_ptr(), ld, ncols, W.data_ptr(), part.data_ptr(),
                                           nparts, C.data_ptr(), sh), "proj")
                _lib.check(L.sg_block_update(code, block, n, Q.data_ptr(), ld, ncols, C.data_ptr(),
                                             W.data_ptr(), sh), "update")
            cholqr2()
            _lib.check(L.sg_lanczos_hblock(block, H.data_ptr(), ld, m, C1.data_ptr(), C2.data_ptr(), R1.data_ptr(),
                                           R2.data_ptr(), Rout.data_ptr(), 1, sh), "hblock")
            _lib.check(L.sg_block_finish(code, block, n, W.data_ptr(), Q.data_ptr(), ld, m + block, Z.data_ptr(),
                                         Zs.data_ptr(), a.data_ptr(), sh), "finish")
            m += block
        # after a thick restart keep need not be a multiple of the block, so
        # the basis ends at m (<= M): the Ritz problem is H[:m, :m]
        Me = m
        Hh = H.cpu().numpy()
        st.raise_if_error("block Lanczos (rank-deficient Krylov block)")
        tr = time.perf_counter()
        ph["cycles"] += tr - tc
        th, Y = np.linalg.eigh(Hh[:Me, :Me])
        Rl = Hh[Me:Me + block, Me - block:Me]
        res = np.linalg.norm(Rl @ Y[Me - block:Me, :], axis=0)
        order = np.argsort(-np.abs(th), kind="stable")
        sel = order[:k]
        anorm = max(float(np.abs(th).max()), 1e-300)
        need = np.where((th[sel] > 0) | (not vec_positive_only), tol_vec, tol_val) * anorm
        worst = float(np.max(res[sel] / need))
        hist.append(float(res[sel].max()))
        tq = time.perf_counter()
        ph["ritz"] += tq - tr
        if worst <= 1.0 or restarts >= max_restarts:
            break
        # FP32 floor: the residuals stopped falling while already within a few
        # hundred FP32 ulps of |A| (slow convergence above that keeps going)
        if (precision == "mixed" and len(hist) >= 6 and min(hist[-3:]) > 0.7 * min(hist[:-3])
                and min(hist) <= FP32_FLOOR * anorm):
            break
        restarts += 1
        kp = order[:keep]
        Yk = torch.from_numpy(np.ascontiguousarray(Y[:, kp])).to(dev)
        _lib.check(L.sg_basis_rotate(code, code, n, Q.data_ptr(), ld, Me, Yk.data_ptr(), keep, keep, Q2.data_ptr(),
                                     ld, sh), "rotate")
        _lib.check(L.sg_block_finish(code, block, n, Z.data_ptr(), Q2.data_ptr(), ld, keep, None, None, None, sh),
                   "finish")
        Q, Q2 = Q2, Q
        Hn = np.zeros((ld, ld))
        Hn[np.arange(keep), np.arange(keep)] = th[kp]
        Bc = Rl @ Y[Me - block:Me, kp]
        Hn[keep:keep + block, :keep] = Bc
        Hn[:keep, keep:keep + block] = Bc.T
        H.copy_(torch.from_numpy(Hn))
        m = keep
        ph["restart"] += time.perf_counter() - tq
    # Ritz vectors (FP64 output), eigenvalues sorted descending like the reference
    sel = order[:k]
    sel = sel[np.argsort(-th[sel], kind="stable")]
    Yk = torch.from_numpy(np.ascontiguousarray(Y[:, sel])).to(dev)
    U = torch.empty(n, k, **f64)
    _lib.check(L.sg_basis_rotate(code, 1, n, Q.data_ptr(), ld, Me, Yk.data_ptr(), k, k, U.data_ptr(), k, sh),
               "rotate")
    evals = th[sel].copy()
    tf = time.perf_counter()
    if refine and precision == "mixed" and k <= 32:
        evals, U = fp64_refine(op, U, k, sh)
    torch.cuda.synchronize(dev)
    ph["refine"] = time.perf_counter() - tf
    beyond = order[k:k + 4]  # Ritz values just outside the wanted set
    info = dict(block_matvecs=n_mv, vector_matvecs=n_mv * block, restarts=restarts, basis=M, keep=keep,
                residuals=res[sel].tolist(), converged=worst <= 1.0, seconds=time.perf_counter() - t0,
                precision=precision, block=block, next_evals=th[beyond].tolist(), phase_seconds=ph)
    return EigenResult(evals, U, info)


def residual_norms(op: GramOperator, U: torch.Tensor, evals) -> np.ndarray:
    """FP64 residuals ||A u_i - λ_i u_i|| of k <= 32 eigenpairs (U: n x k on
    the device), from one FP64 block matvec: the accuracy check of a result
    that has no CPU oracle at its size."""
    L = _lib.load()
    n, dev = op.n, op.a.device
    k = int(U.shape[1])
    kb = 32
    if k > kb:
        raise ValueError("residual_norms supports k <= 32")
    sh = torch.cuda.current_stream(dev).cuda_stream
    f64 = dict(dtype=torch.float64, device=dev)
    Up = torch.zeros(n, kb, **f64)
    Up[:, :k] = U.to(torch.float64)
    Zs, W = torch.empty(n, kb, **f64), torch.empty(n, kb, **f64)
    T = torch.empty(op.m, kb, **f64)
    _lib.check(L.sg_block_finish(1, kb, n, Up.data_ptr(), None, 0, 0, None, Zs.data_ptr(), op.a.data_ptr(), sh),
               "scale")
    op.apply(1, kb, Up, Zs, T, W, sh)
    lam = torch.as_tensor(np.asarray(evals, dtype=np.float64), device=dev)
    R = W[:, :k] - Up[:, :k] * lam
    return torch.linalg.vector_norm(R, dim=0).cpu().numpy()


def fp64_refine(op: GramOperator, U: torch.Tensor, k: int, stream: int):
    """Final FP64 residual-correction sweep of mixed-precision Ritz pairs.

    U (n x k, FP64) spans the converged FP32 Ritz vectors.  One FP64 block
    matvec A U (FP64 SpMM, block 32) and FP64 Rayleigh-Ritz on span(U)
    (Gram matrix G = UᵀU, H = Uᵀ A U, generalized eigenproblem H y = θ G y by
    Cholesky) give eigenvalues with error O(angle²), i.e. at FP64 level, and
    re-rotate the vectors inside the subspace.  Returns (θ descending, U').
    """
    L = _lib.load()
    n, dev = op.n, op.a.device
    kb = 32
    if k > kb:
        raise ValueError("refinement supports k <= 32")
    f64 = dict(dtype=torch.float64, device=dev)
    Up = torch.zeros(n, kb, **f64)
    eye = torch.eye(k, dtype=torch.float64).to(dev)
    _lib.check(L.sg_basis_rotate(1, 1, n, U.data_ptr(), k, k, eye.data_ptr(), k, k, Up.data_ptr(), kb, stream),
               "copy")
    nparts = int(L.sg_proj_parts())
    part = torch.empty(nparts * kb * kb, **f64)
    G = torch.empty(kb * kb, **f64)
    Hm = torch.empty(kb * kb, **f64)
    Zs, W = torch.empty(n, kb, **f64), torch.empty(n, kb, **f64)
    T = torch.empty(op.m, kb, **f64)
    _lib.check(L.sg_block_proj(1, kb, n, Up.data_ptr(), kb, kb, Up.data_ptr(), part.data_ptr(), nparts,
                               G.data_ptr(), stream), "gram")
    _lib.check(L.sg_block_finish(1, kb, n, Up.data_ptr(), None, 0, 0, None, Zs.data_ptr(), op.a.data_ptr(), stream),
               "scale")
    op.apply(1, kb, Up, Zs, T, W, stream)
    _lib.check(L.sg_block_proj(1, kb, n, Up.data_ptr(), kb, kb, W.data_ptr(), part.data_ptr(), nparts,
                               Hm.data_ptr(), stream), "rayleigh quotient")
    Gk = G.cpu().numpy().reshape(kb, kb)[:k, :k]
    Hk = Hm.cpu().numpy().reshape(kb, kb)[:k, :k]
    Hk = 0.5 * (Hk + Hk.T)
    Rc = np.linalg.cholesky(0.5 * (Gk + Gk.T)).T      # G = Rᵀ R
    Ri = np.linalg.inv(Rc)
    th, Zr = np.linalg.eigh(Ri.T @ Hk @ Ri)
    Y = Ri @ Zr
    order = np.argsort(-th, kind="stable")
    Yt = torch.from_numpy(np.ascontiguousarray(Y[:, order])).to(dev)
    Un = torch.empty(n, k, **f64)
    _lib.check(L.sg_basis_rotate(1, 1, n, Up.data_ptr(), kb, k, Yt.data_ptr(), k, k, Un.data_ptr(), k, stream),
               "rotate")
    return th[order].copy(), Un


def _dense_small(op: GramOperator, k: int, code: int, tdt, block: int) -> EigenResult:
    """Tiny problems: apply A to the identity on the GPU and solve densely."""
    L = _lib.load()
    n, dev = op.n, op.a.device
    sh = torch.cuda.current_stream(dev).cuda_stream
    kw = dict(dtype=tdt, device=dev)
    w2, a, dinv = op.scales(code)
    A = np.zeros((n, n))
    Z, Zs, W = (torch.zeros(n, block, **kw) for _ in range(3))
    T = torch.empty(op.m, block, **kw)
    for c0 in range(0, n, block):
        Z.zero_()
        cols = min(block, n - c0)
        Z[torch.arange(c0, c0 + cols, device=dev), torch.arange(cols, device=dev)] = 1
        _lib.check(L.sg_block_finish(code, block, n, Z.data_ptr(), None, 0, 0, None, Zs.data_ptr(), a.data_ptr(),
                                     sh), "finish")
        op.apply(code, block, Z, Zs, T, W, sh)
        A[:, c0:c0 + cols] = W[:, :cols].double().cpu().numpy()
    A = 0.5 * (A + A.T)
    th, Y = np.linalg.eigh(A)
    order = np.argsort(-np.abs(th), kind="stable")[:k]
    order = order[np.argsort(-th[order], kind="stable")]
    U = torch.from_numpy(np.ascontiguousarray(Y[:, order])).to(dev)
    return EigenResult(th[order].copy(), U, dict(dense=True, n=n, block_matvecs=(n + block - 1) // block,
                                                 restarts=0, converged=True, residuals=[0.0]))
