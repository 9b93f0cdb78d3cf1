"""Many independent datasets embedded together on one GPU.

The datasets' matrices are stacked block-diagonally into one CSR; the Gram
SpMM passes are then single launches over all datasets, and the dense block
operations of the Krylov-Schur iteration run as batched kernels
(``csrc/batched.cu``) with the dataset boundaries as arguments.  Every restart
cycle of block expansions (fixed kernel arguments) is captured once in a CUDA
graph and replayed; between cycles the host solves the datasets' small
Rayleigh-Ritz problems in a thread pool (LAPACK releases the GIL), tests
convergence per dataset and freezes converged ones.

Each dataset's embedding is mathematically the same as a separate
``snap.tl.spectral`` call: IDF per dataset (``sg_bidf``), normalisation and
degrees are row/column local, and the eigenproblems never couple.
"""
from __future__ import annotations

import math
import time
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass

import numpy as np
import torch

from . import _eigen, _lib
from ._hostblas import blas_threads
from ._binning import DeviceCSR

_DT = {"mixed": (0, torch.float32), "fp64": (1, torch.float64)}


@dataclass
class BatchedOperator:
    D: int
    roff: np.ndarray          # int64 [D+1] row offsets
    coff: np.ndarray          # int64 [D+1] column offsets
    op: _eigen.GramOperator   # on the stacked matrix
    timings: dict | None = None  # seconds of the build phases


def stack(mats: list[DeviceCSR]) -> tuple[DeviceCSR, np.ndarray, np.ndarray]:
    """Block-diagonal stacking (row pointers and column indices offset)."""
    dev = mats[0].indptr.device
    roff = np.zeros(len(mats) + 1, dtype=np.int64)
    coff = np.zeros(len(mats) + 1, dtype=np.int64)
    nnz_off = 0
    ptrs, idxs, vals = [], [], []
    for d, c in enumerate(mats):
        n, m = c.shape
        roff[d + 1] = roff[d] + n
        coff[d + 1] = coff[d] + m
        ptrs.append(c.indptr[:-1] + nnz_off)
        idxs.append(c.indices + int(coff[d]))
        if c.data is not None:
            vals.append(c.data)
        nnz_off += c.nnz
    if vals and len(vals) != len(mats):
        vals = [c.data if c.data is not None else torch.ones(c.nnz, dtype=torch.float32, device=dev) for c in mats]
    ptrs.append(torch.tensor([nnz_off], dtype=torch.int64, device=dev))
    S = DeviceCSR(torch.cat(ptrs), torch.cat(idxs).to(torch.int32), torch.cat(vals) if vals else None,
                  (int(roff[-1]), int(coff[-1])))
    return S, roff, coff


def build_batched_operator(mats: list[DeviceCSR]) -> BatchedOperator:
    """Stacked operator of the datasets.  The CSC of the block-diagonal stack
    is the concatenation of the datasets' own CSCs (row indices offset by the
    dataset's first row, column pointers by its first nonzero), so each
    dataset is transposed on its own: a transpose of the stack would walk
    every row once per 16,384-column panel of all datasets together."""
    L = _lib.lib()
    dev = mats[0].indptr.device
    tm = {}
    t0 = time.perf_counter()
    S, roff, coff = stack(mats)
    torch.cuda.synchronize(dev)
    tm["stack"] = time.perf_counter() - t0
    D = len(mats)
    n, m = S.shape
    sh = torch.cuda.current_stream(dev).cuda_stream
    colptr = torch.empty(m + 1, dtype=torch.int64, device=dev)
    rowidx = torch.empty(max(S.nnz, 1), dtype=torch.int32, device=dev)
    cval = torch.empty(max(S.nnz, 1), dtype=torch.float32, device=dev) if S.data is not None else None
    z0 = 0
    for d, c in enumerate(mats):
        cp, ri, cv = _eigen.transpose(c, sh)
        nz = c.nnz
        c0, c1 = int(coff[d]), int(coff[d + 1])
        torch.add(cp[:-1], z0, out=colptr[c0:c1])
        torch.add(ri, int(roff[d]), out=rowidx[z0:z0 + nz])
        if cval is not None:
            cval[z0:z0 + nz].copy_(cv if cv is not None else torch.ones(nz, dtype=torch.float32, device=dev))
        z0 += nz
        del cp, ri, cv
    colptr[m] = z0
    torch.cuda.synchronize(dev)
    tm["transpose"] = time.perf_counter() - t0 - tm["stack"]
    # IDF per dataset (its own cell count), then the stacked operator
    roff_t = torch.from_numpy(roff).to(dev)
    coff_t = torch.from_numpy(coff).to(dev)
    mm = torch.empty(2 * D, dtype=torch.int64, device=dev)
    w = torch.empty(m, dtype=torch.float64, device=dev)
    _lib.check(L.sg_bidf(m, colptr.data_ptr(), D, coff_t.data_ptr(), roff_t.data_ptr(), mm.data_ptr(), w.data_ptr(),
                         sh), "sg_bidf")
    op = _eigen.build_operator(S, w, csc=(colptr, rowidx[:S.nnz], cval[:S.nnz] if cval is not None else None))
    torch.cuda.synchronize(dev)
    tm["operator"] = time.perf_counter() - t0 - tm["stack"] - tm["transpose"]
    return BatchedOperator(D, roff, coff, op, tm)


def _cta_partition(roff: np.ndarray, target: int):
    """CTAs over the rows of each dataset (never crossing a dataset)."""
    ds, r0, r1, first = [], [], [], [0]
    for d in range(len(roff) - 1):
        n = int(roff[d + 1] - roff[d])
        c = max(1, int(round(n / target)))
        for j in range(c):
            ds.append(d)
            r0.append(int(roff[d]) + n * j // c)
            r1.append(int(roff[d]) + n * (j + 1) // c)
        first.append(len(ds))
    return (np.array(ds, np.int32), np.array(r0, np.int64), np.array(r1, np.int64), np.array(first, np.int32))


@dataclass
class BatchedResult:
    evals: list            # per dataset: k eigenvalues (descending)
    evecs: torch.Tensor    # stacked (sum n) x k FP64
    roff: np.ndarray
    info: dict


def eigsh_lm_batched(bop: BatchedOperator, k: int, *, precision: str = "mixed", block: int = 8,
                     max_basis: int | None = None, keep: int | None = None, tol_vec: float = _eigen.TOL_VEC,
                     tol_val: float = 1e-6, seed: int = 0, max_restarts: int = 200, use_graphs: bool = True,
                     threads: int = 16, refine: bool = True) -> BatchedResult:
    L = _lib.lib()
    code, tdt = _DT[precision]
    op, D, roff = bop.op, bop.D, bop.roff
    dev = op.a.device
    n_tot = op.n
    nmin = int(np.min(np.diff(roff)))
    if k < 1 or k >= nmin:
        raise ValueError("every dataset needs more than k cells")
    M0, keep0 = _eigen._default_basis(k, block, nmin)
    M = min(int(max_basis or M0), (nmin - block) // block * block)
    keep = min(int(keep or keep0), M - block)
    if keep < k:
        raise ValueError("the smallest dataset is too small for the requested k")
    ld = M + block
    kw = dict(dtype=tdt, device=dev)
    f64 = dict(dtype=torch.float64, device=dev)
    Qa, Qb = torch.empty(n_tot, ld, **kw), torch.empty(n_tot, ld, **kw)
    Z, Zs, W = (torch.empty(n_tot, block, **kw) for _ in range(3))
    T = torch.empty(op.m, block, **kw)
    ds_np, r0_np, r1_np, first_np = _cta_partition(roff, max(256, n_tot // (4 * 152)))
    ncta = int(ds_np.shape[0])
    cta_ds, cta_r0, cta_r1, ds_cta = (torch.from_numpy(x).to(dev) for x in (ds_np, r0_np, r1_np, first_np))
    roff_t = torch.from_numpy(roff).to(dev)
    coff_t = torch.from_numpy(bop.coff).to(dev)
    active = torch.ones(D, dtype=torch.int32, device=dev)
    # SpMM row masks (cells, features) of frozen datasets
    op.row_mask = torch.ones(n_tot, dtype=torch.uint8, device=dev)
    op.col_mask = torch.ones(op.m, dtype=torch.uint8, device=dev)
    cstride = ld * block
    part = torch.empty(ncta * 512 * block, **f64)
    C1, C2 = torch.empty(D * cstride, **f64), torch.empty(D * cstride, **f64)
    G = torch.empty(D * block * block, **f64)
    R1, R2, Rinv, Rout = (torch.empty(D * block * block, **f64) for _ in range(4))
    H = torch.zeros(D, ld, ld, **f64)
    st = _lib.DeviceStatus(dev)
    w2, a, dinv = op.scales(code)
    chk = _lib.check

    def cholqr2(sh):
        for R in (R1, R2):
            chk(L.sg_bblock_cholqr(code, block, n_tot, D, roff_t.data_ptr(), active.data_ptr(), ncta,
                                   ds_cta.data_ptr(), cta_ds.data_ptr(), cta_r0.data_ptr(), cta_r1.data_ptr(),
                                   W.data_ptr(),
                                   part.data_ptr(), G.data_ptr(), R.data_ptr(), Rinv.data_ptr(), st.status_ptr,
                                   None, sh), "batched cholqr")

    def expand(Q, m0, sh):
        m = m0
        while m + block <= M:
            op.apply(code, block, Z, Zs, T, W, sh)
            ncols = m + block
            for C in (C1, C2):
                chk(L.sg_bblock_proj(code, block, D, ncta, ds_cta.data_ptr(), cta_ds.data_ptr(), active.data_ptr(),
                                     cta_r0.data_ptr(), cta_r1.data_ptr(), Q.data_ptr(), ld, ncols, W.data_ptr(),
                                     part.data_ptr(), C.data_ptr(), cstride, sh), "batched proj")
                chk(L.sg_bblock_update(code, block, n_tot, D, roff_t.data_ptr(), active.data_ptr(), Q.data_ptr(), ld,
                                       ncols, C.data_ptr(), cstride, W.data_ptr(), sh), "batched update")
            cholqr2(sh)
            chk(L.sg_blanczos_hblock(block, D, active.data_ptr(), H.data_ptr(), ld, m, C1.data_ptr(), C2.data_ptr(),
                                     cstride, R1.data_ptr(), R2.data_ptr(), Rout.data_ptr(), sh), "batched hblock")
            chk(L.sg_block_finish(code, block, n_tot, W.data_ptr(), Q.data_ptr(), ld, m + block, Z.data_ptr(),
                                  Zs.data_ptr(), a.data_ptr(), sh), "finish")
            m += block
        return m

    t0 = time.perf_counter()
    sh0 = torch.cuda.current_stream(dev).cuda_stream
    chk(L.sg_fill_random(code, n_tot * block, int(seed) & 0xFFFFFFFFFFFFFFFF, W.data_ptr(), sh0), "fill")
    cholqr2(sh0)
    chk(L.sg_block_finish(code, block, n_tot, W.data_ptr(), Qa.data_ptr(), ld, 0, Z.data_ptr(), Zs.data_ptr(),
                          a.data_ptr(), sh0), "finish")
    if (code, block) not in op.variants:  # tune before any capture (the tuner synchronises)
        _eigen.tune_spmm(op, code, block, Z, Zs, T, W, sh0)
    graphs = {}

    def run_cycle(Q, m0):
        key = (Q.data_ptr(), m0)
        if not use_graphs:
            return expand(Q, m0, torch.cuda.current_stream(dev).cuda_stream)
        if key not in graphs:
            g = torch.cuda.CUDAGraph()
            torch.cuda.synchronize(dev)
            with torch.cuda.graph(g, capture_error_mode="relaxed"):
                expand(Q, m0, torch.cuda.current_stream(dev).cuda_stream)
            graphs[key] = g
        graphs[key].replay()
        return m0 + (M - m0) // block * block  # where expand() stops

    Q, Q2 = Qa, Qb
    m0 = 0
    n_mv = 0
    restarts = 0
    conv = np.zeros(D, bool)
    # settled: converged and rotated once since, so its k wanted Ritz vectors
    # are basis columns 0..k-1 (largest magnitude first) and later restarts
    # leave its first `keep` columns in place
    settled = np.zeros(D, bool)
    Ys = [None] * D
    pool = ThreadPoolExecutor(max_workers=threads)
    ph = dict(cycles=0.0, ritz=0.0, restart=0.0, refine=0.0)
    while True:
        tc = time.perf_counter()
        Me = run_cycle(Q, m0)
        n_mv += (Me - m0) // block
        Hh = H.cpu().numpy()
        st.raise_if_error("batched block Lanczos (rank-deficient Krylov block)")
        tr = time.perf_counter()
        ph["cycles"] += tr - tc

        def ritz(d):
            th, Y = np.linalg.eigh(Hh[d, :Me, :Me])
            Rl = Hh[d, Me:Me + block, Me - block:Me]
            res = np.linalg.norm(Rl @ Y[Me - block:Me, :], axis=0)
            order = np.argsort(-np.abs(th), kind="stable")
            sel = order[:k]
            anorm = max(float(np.abs(th).max()), 1e-300)
            need = np.where(th[sel] > 0, tol_vec, tol_val) * anorm
            return th, Y, Rl, order, float(np.max(res[sel] / need))

        live = [d for d in range(D) if not conv[d]]  # converged datasets keep their last Ritz pairs
        with blas_threads(1):  # one LAPACK thread per pool thread
            out = list(pool.map(ritz, live))
        for d, (th, Y, Rl, order, worst) in zip(live, out):
            Ys[d] = (th, Y, Rl, order)
            if worst <= 1.0:
                conv[d] = True
        tq = time.perf_counter()
        ph["ritz"] += tq - tr
        if conv.all() or restarts >= max_restarts:
            break
        restarts += 1
        # thick restart of every dataset (converged ones keep their basis)
        Ybuf = np.zeros((D, Me, keep))
        Hn = np.zeros((D, ld, ld))
        for d in range(D):
            if settled[d]:
                Ybuf[d, np.arange(keep), np.arange(keep)] = 1.0
                continue
            th, Y, Rl, order = Ys[d]
            kp = order[:keep]
            Ybuf[d] = Y[:, kp]
            Hn[d, np.arange(keep), np.arange(keep)] = th[kp]
            Bc = Rl @ Y[Me - block:Me, kp]
            Hn[d, keep:keep + block, :keep] = Bc
            Hn[d, :keep, keep:keep + block] = Bc.T
            if conv[d]:
                settled[d] = True
        Yt = torch.from_numpy(Ybuf).to(dev)
        chk(L.sg_bbasis_rotate(code, code, ncta, cta_ds.data_ptr(), cta_r0.data_ptr(), cta_r1.data_ptr(), Q.data_ptr(),
                               ld, Me, Yt.data_ptr(), keep, Me * keep, keep, Q2.data_ptr(), ld, sh0), "batched rotate")
        chk(L.sg_block_finish(code, block, n_tot, Z.data_ptr(), Q2.data_ptr(), ld, keep, None, None, None, sh0),
            "finish")
        Q, Q2 = Q2, Q
        H.copy_(torch.from_numpy(Hn))
        active.copy_(torch.from_numpy((~conv).astype(np.int32)))
        chk(L.sg_bmask(n_tot, D, roff_t.data_ptr(), active.data_ptr(), op.row_mask.data_ptr(), sh0), "mask")
        chk(L.sg_bmask(op.m, D, coff_t.data_ptr(), active.data_ptr(), op.col_mask.data_ptr(), sh0), "mask")
        m0 = keep
        ph["restart"] += time.perf_counter() - tq
    pool.shutdown()
    op.row_mask = op.col_mask = None
    Ybuf = np.zeros((D, Me, k))
    ev_out = []
    for d in range(D):
        th, Y, Rl, order = Ys[d]
        sel = order[:k]
        vals = th[sel]
        desc = np.argsort(-vals, kind="stable")
        if settled[d]:  # wanted vectors are columns 0..k-1 in the order of `sel`
            Ybuf[d, desc, np.arange(k)] = 1.0
        else:
            Ybuf[d] = Y[:, sel[desc]]
        ev_out.append(vals[desc].copy())
    Yt = torch.from_numpy(Ybuf).to(dev)
    U = torch.empty(n_tot, k, **f64)
    chk(L.sg_bbasis_rotate(code, 1, ncta, cta_ds.data_ptr(), cta_r0.data_ptr(), cta_r1.data_ptr(), Q.data_ptr(), ld,
                           Me, Yt.data_ptr(), k, Me * k, k, U.data_ptr(), k, sh0), "batched rotate")
    tf = time.perf_counter()
    if refine and precision == "mixed" and k <= 32:
        ev_out, U = _refine_batched(op, D, k, U, ncta, cta_ds, cta_r0, cta_r1, ds_cta, sh0)
    torch.cuda.synchronize(dev)
    ph["refine"] = time.perf_counter() - tf
    info = dict(block_matvecs=n_mv, restarts=restarts, converged=int(conv.sum()), datasets=D, basis=M, keep=keep,
                graphs=len(graphs), seconds=time.perf_counter() - t0, phase_seconds=ph)
    return BatchedResult(ev_out, U, roff, info)


def _refine_batched(op, D, k, U, ncta, cta_ds, cta_r0, cta_r1, ds_cta, sh):
    """FP64 residual-correction sweep of every dataset (see _eigen.fp64_refine):
    one stacked FP64 SpMM, per-dataset Gram and Rayleigh quotients, host
    generalized eigenproblems, per-dataset rotation."""
    L = _lib.load()
    chk = _lib.check
    n, dev = op.n, op.a.device
    kb = 32
    f64 = dict(dtype=torch.float64, device=dev)
    Up = torch.zeros(n, kb, **f64)
    eye = torch.eye(k, dtype=torch.float64).to(dev)
    chk(L.sg_basis_rotate(1, 1, n, U.data_ptr(), k, k, eye.data_ptr(), k, k, Up.data_ptr(), kb, sh), "copy")
    part = torch.empty(ncta * kb * kb, **f64)
    G = torch.empty(D * kb * kb, **f64)
    Hm = torch.empty(D * kb * kb, **f64)
    Zs, W = torch.empty(n, kb, **f64), torch.empty(n, kb, **f64)
    T = torch.empty(op.m, kb, **f64)
    for Wm, out in ((Up, G), (None, Hm)):
        if Wm is None:
            chk(L.sg_block_finish(1, kb, n, Up.data_ptr(), None, 0, 0, None, Zs.data_ptr(), op.a.data_ptr(), sh),
                "scale")
            op.apply(1, kb, Up, Zs, T, W, sh)
            Wm = W
        chk(L.sg_bblock_proj(1, kb, D, ncta, ds_cta.data_ptr(), cta_ds.data_ptr(), None, cta_r0.data_ptr(),
                             cta_r1.data_ptr(), Up.data_ptr(), kb, kb, Wm.data_ptr(), part.data_ptr(), out.data_ptr(),
                             kb * kb, sh), "batched proj")
    Gh = G.cpu().numpy().reshape(D, kb, kb)[:, :k, :k]
    Hh = Hm.cpu().numpy().reshape(D, kb, kb)[:, :k, :k]
    Ybuf = np.zeros((D, kb, k))
    evs = []
    for d in range(D):
        Gk = 0.5 * (Gh[d] + Gh[d].T)
        Hk = 0.5 * (Hh[d] + Hh[d].T)
        Ri = np.linalg.inv(np.linalg.cholesky(Gk).T)
        th, Zr = np.linalg.eigh(Ri.T @ Hk @ Ri)
        o = np.argsort(-th, kind="stable")
        Ybuf[d, :k] = (Ri @ Zr)[:, o]
        evs.append(th[o].copy())
    Yt = torch.from_numpy(Ybuf).to(dev)
    Un = torch.empty(n, k, **f64)
    chk(L.sg_bbasis_rotate(1, 1, ncta, cta_ds.data_ptr(), cta_r0.data_ptr(), cta_r1.data_ptr(), Up.data_ptr(), kb, kb,
                           Yt.data_ptr(), k, kb * k, k, Un.data_ptr(), k, sh), "batched rotate")
    return evs, Un


def spectral_batched(mats, n_comps: int = 30, *, precision: str = "auto", block: int = 8, weighted_by_sd=True,
                     **kw):
    """Embed many datasets together; returns a list of (evals, X_spectral) per
    dataset with the same post-processing as ``snap.tl.spectral``.
    precision='auto' runs FP64 when every dataset is below the single-call
    threshold (``tools.AUTO_FP64_CELLS``), mixed otherwise."""
    from .tools import AUTO_FP64_CELLS, csr_to_device
    dev = torch.device("cuda", torch.cuda.current_device())
    mats = [csr_to_device(X, dev) for X in mats]
    if precision == "auto":
        precision = "fp64" if max(c.shape[0] for c in mats) < AUTO_FP64_CELLS else "mixed"
    bop = build_batched_operator(mats)
    res = eigsh_lm_batched(bop, n_comps, precision=precision, block=block, **kw)
    out = []
    for d in range(bop.D):
        ev = res.evals[d]
        E = res.evecs[int(bop.roff[d]):int(bop.roff[d + 1])].cpu().numpy()
        if weighted_by_sd:
            idx = [i for i in range(ev.shape[0]) if ev[i] > 0]
            ev = ev[idx]
            E = E[:, idx] * np.sqrt(ev)
        out.append((ev, E))
    return out


def embed_concurrent(mats, n_comps: int = 30, *, precision: str = "mixed", block: int | None = 8,
                     streams: int = 8, **kw) -> list:
    """Embed independent datasets concurrently: each dataset is one
    build_operator + sg_lanczos solve on its own CUDA stream, from a pool of
    ``streams`` host threads (sg_lanczos runs its whole restart loop in the
    library with the GIL released, so the threads' launches and their
    per-restart decisions overlap).  Datasets start largest first; each
    leaves as soon as its own solve has converged, so small datasets never
    wait for large ones and the GPU keeps several solves in flight.

    Returns the list of EigenResult, in the order of ``mats``; each equals a
    separate eigsh_lm of that dataset (same kernels, same arithmetic).
    """
    dev = torch.device("cuda", torch.cuda.current_device())
    order = sorted(range(len(mats)), key=lambda d: -int(mats[d].nnz))
    pool_streams = [torch.cuda.Stream(device=dev) for _ in range(max(1, streams))]
    free = list(range(len(pool_streams)))
    import threading
    lock = threading.Lock()
    out: list = [None] * len(mats)
    # the caller's work on its current stream precedes every solve
    start = torch.cuda.Event()
    start.record(torch.cuda.current_stream(dev))

    def run(d):
        with lock:
            si = free.pop()
        s = pool_streams[si]
        try:
            torch.cuda.set_device(dev)
            s.wait_event(start)
            with torch.cuda.stream(s):
                op = _eigen.build_operator(mats[d])
                out[d] = _eigen.eigsh_lm(op, n_comps, precision=precision, block=block, stream=s, **kw)
                del op
            s.synchronize()
        finally:
            with lock:
                free.append(si)

    with ThreadPoolExecutor(max_workers=len(pool_streams)) as ex:
        for f in [ex.submit(run, d) for d in order]:
            f.result()
    return out
