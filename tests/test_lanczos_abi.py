"""The one-call eigensolver sg_lanczos and its GPU Rayleigh-Ritz step
sg_sym_eig, called through the C ABI.

sg_sym_eig is checked against LAPACK (numpy.linalg.eigh) on random symmetric
matrices, on matrices with exactly repeated and tightly clustered eigenvalues
and on the arrowhead + block-tridiagonal shape the thick restart produces, up
to the 640 x 640 limit: eigenvalues within 1e-12 ‖A‖, residuals
‖A y - λ y‖ within 1e-11 ‖A‖, the returned vectors orthonormal to 1e-10.

sg_lanczos replaces the reference's eigsh call (snapatac2-python/src/
embedding.rs:155-188); it is called directly with an operator built by
build_operator and compared with the oracle's ARPACK result (eigenvalues
1e-5 relative, principal angles 1e-4 rad per cluster) and with the earlier
solver that ran the Rayleigh-Ritz step on the host.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import spectral as osp
from snapatac2_gb300 import synthetic as syn
from test_spectral import check_eigs


def _sym_eig(A, p, q):
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    dev = torch.device("cuda")
    n = A.shape[0]
    At = torch.from_numpy(np.ascontiguousarray(A, dtype=np.float64)).to(dev)
    nw = n if p + q >= n else p + q
    nb = int(L.sg_sym_eig_work_bytes(n, p, q))
    work = torch.empty(nb, dtype=torch.uint8, device=dev)
    ev = torch.empty(nw, dtype=torch.float64, device=dev)
    vecs = torch.empty(nw, n, dtype=torch.float64, device=dev)
    rc = L.sg_sym_eig(n, At.data_ptr(), n, p, q, ev.data_ptr(), vecs.data_ptr(), work.data_ptr(), nb,
                      torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0
    return ev.cpu().numpy(), vecs.cpu().numpy()


def _check_sym(A, p, q):
    n = A.shape[0]
    ev, Y = _sym_eig(A, p, q)
    w = np.linalg.eigvalsh(A)
    ranks = np.arange(n) if p + q >= n else np.concatenate([np.arange(q), np.arange(n - p, n)])
    nrm = max(np.abs(w).max(), 1e-300)
    assert np.all(np.abs(ev - w[ranks]) <= 1e-12 * nrm), np.abs(ev - w[ranks]).max() / nrm
    R = A @ Y.T - Y.T * ev
    assert np.linalg.norm(R, axis=0).max() <= 1e-11 * nrm
    G = Y @ Y.T
    assert np.abs(G - np.eye(len(ev))).max() <= 1e-10


def _restart_shape(n, keep, b, rng):
    """diag(θ) of the kept pairs, a b-wide coupling block, then block
    tridiagonal blocks of width b (the matrix a thick restart expands)."""
    H = np.zeros((n, n))
    H[np.arange(keep), np.arange(keep)] = np.sort(rng.uniform(-0.3, 1.0, keep))[::-1]
    B = rng.standard_normal((b, keep)) * 1e-3
    H[keep:keep + b, :keep] = B
    H[:keep, keep:keep + b] = B.T
    for s in range(keep, n, b):
        e = min(s + b, n)
        D = rng.standard_normal((e - s, e - s)) * 0.1
        H[s:e, s:e] = 0.5 * (D + D.T)
        if e < n:
            e2 = min(e + b, n)
            R = np.triu(rng.standard_normal((e2 - e, e - s))) * 0.05
            H[e:e2, s:e] = R
            H[s:e, e:e2] = R.T
    return H


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 200, 576, 640])
def test_sym_eig_random_matrices(n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n))
    _check_sym(0.5 * (X + X.T), n, n)
    if n > 20:
        _check_sym(0.5 * (X + X.T), 7, 5)  # subsets at both ends


@pytest.mark.gpu
def test_sym_eig_repeated_and_clustered_eigenvalues():
    rng = np.random.default_rng(3)
    n = 150
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.concatenate([np.full(20, 0.5), 0.9 + 1e-9 * np.arange(15), rng.uniform(-1, 1, n - 35)])
    A = (Q * lam) @ Q.T
    _check_sym(0.5 * (A + A.T), n, n)
    _check_sym(np.diag(np.repeat([1.0, 2.0, 3.0], 10)), 30, 30)  # already diagonal, degenerate


@pytest.mark.gpu
@pytest.mark.parametrize("n,keep,b", [(200, 80, 8), (576, 94, 32), (120, 46, 4)])
def test_sym_eig_restart_shape(n, keep, b):
    rng = np.random.default_rng(n + keep)
    H = _restart_shape(n, keep, b, rng)
    _check_sym(H, keep + 4, keep + 4)


def _operator(n=3000, m=60000, nnz=400, seed=9):
    import torch
    from snapatac2_gb300 import _eigen
    from snapatac2_gb300._binning import DeviceCSR
    B = syn.binary_csr(n, m, nnz_per_cell=nnz, seed=seed)
    X = sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)
    dev = torch.device("cuda")
    csr = DeviceCSR(torch.from_numpy(B.indptr).to(dev), torch.from_numpy(B.indices).to(dev), None, B.shape)
    return X, _eigen.build_operator(csr)


def _gram_op(op):
    from snapatac2_gb300 import _lib
    p = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    return _lib.GramOp(op.n, op.m, p(op.csr.indptr), p(op.csr.indices), None, p(op.colptr), p(op.rowidx), None,
                       p(op.w2), p(op.a), p(op.dinv), p(op.w2_32), p(op.a32), p(op.dinv32), None, None)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,block", [(0, 8), (1, 8), (0, 16), (1, 4)])
def test_sg_lanczos_direct_call_matches_oracle(precision, block):
    """ctypes call of sg_lanczos with the operator's device pointers; no
    Python driver in between."""
    import torch
    from snapatac2_gb300 import _lib
    X, op = _operator()
    L = _lib.lib()
    n, m, k = op.n, op.m, 30
    gop = _gram_op(op)
    opts = _lib.LanczosOpts()
    opts.vec_positive_only = 1
    opts.refine = 1
    opts.max_restarts = -1
    opts.variant_t = opts.variant_x = opts.refine_variant_t = opts.refine_variant_x = -1
    nb = int(L.sg_lanczos_work_bytes(precision, block, k, n, m, 0, 0))
    assert nb > 0
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    evals = np.empty(k)
    res = np.empty(k)
    U = torch.empty(n, k, dtype=torch.float64, device="cuda")
    info = _lib.LanczosInfo()
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.sg_lanczos(ctypes.byref(gop), precision, block, k, 0, ctypes.byref(opts), work.data_ptr(), nb,
                      evals.ctypes.data, U.data_ptr(), res.ctypes.data, ctypes.byref(info), status.data_ptr(),
                      torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0 and info.converged == 1
    assert np.all(np.diff(evals) <= 0)  # descending like the reference
    assert info.block_matvecs > 0 and info.kernel_launches > info.block_matvecs
    ev_ref, U_ref = osp.eigen(*osp.operator(X), k, 0)
    check_eigs(evals, U.cpu().numpy(), ev_ref, U_ref)


@pytest.mark.gpu
def test_sg_lanczos_null_options_take_the_defaults():
    import torch
    from snapatac2_gb300 import _lib
    X, op = _operator(n=2500, m=50000, nnz=350, seed=4)
    L = _lib.lib()
    k = 20
    gop = _gram_op(op)
    nb = int(L.sg_lanczos_work_bytes(1, 8, k, op.n, op.m, 0, 0))
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    evals = np.empty(k)
    U = torch.empty(op.n, k, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.sg_lanczos(ctypes.byref(gop), 1, 8, k, 0, None, work.data_ptr(), nb, evals.ctypes.data, U.data_ptr(),
                      None, None, st.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0
    ev_ref, U_ref = osp.eigen(*osp.operator(X), k, 0)
    # NULL options: every returned vector converged to the vector bar
    check_eigs(evals, U.cpu().numpy(), ev_ref, U_ref, positive_only=False)


@pytest.mark.gpu
def test_sg_lanczos_matches_host_ritz_driver():
    from snapatac2_gb300 import _eigen
    X, op = _operator(n=4000, m=60000, nnz=500, seed=21)
    a = _eigen.eigsh_lm(op, 30, precision="fp64", block=8)
    b = _eigen.eigsh_lm_host_ritz(op, 30, precision="fp64", block=8)
    assert a.info["converged"] and b.info["converged"]
    check_eigs(a.evals, a.evecs.cpu().numpy(), b.evals, b.evecs.cpu().numpy(), rtol=1e-9, angle=1e-6)


@pytest.mark.gpu
def test_sg_lanczos_refuses_bad_arguments():
    import torch
    from snapatac2_gb300 import _lib
    _, op = _operator(n=600, m=20000, nnz=200, seed=2)
    L = _lib.lib()
    gop = _gram_op(op)
    evals = np.empty(10)
    U = torch.empty(op.n, 10, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    sh = torch.cuda.current_stream().cuda_stream
    nb = int(L.sg_lanczos_work_bytes(0, 8, 10, op.n, op.m, 0, 0))
    work = torch.empty(nb, dtype=torch.uint8, device="cuda")
    call = lambda block, k, nbytes: L.sg_lanczos(  # noqa: E731
        ctypes.byref(gop), 0, block, k, 0, None, work.data_ptr(), nbytes, evals.ctypes.data, U.data_ptr(), None,
        None, st.data_ptr(), sh)
    assert call(6, 10, nb) == _lib.SG_ERR_ARG        # block not 4/8/16/32
    assert call(8, 0, nb) == _lib.SG_ERR_ARG         # k < 1
    assert call(8, 10, nb - 256) == _lib.SG_ERR_CAP  # workspace too small
    assert int(L.sg_lanczos_work_bytes(0, 32, 30, 10**6, 5 * 10**5, 640, 0)) == -1  # Ritz problem above 640


@pytest.mark.gpu
def test_block_autotuner_choice_is_cached_and_solves_to_the_oracle():
    from snapatac2_gb300 import _eigen
    X, op = _operator(n=5000, m=60000, nnz=500, seed=33)
    b = _eigen.choose_block(op, 30, "mixed")
    assert b in (4, 8, 16, 32)
    key = _eigen._shape_class(op, 0, 30)
    best, pred = _eigen._BLOCK_CHOICE[key]
    assert best == b and b in pred and all(v > 0 for v in pred.values())
    assert _eigen.choose_block(op, 30, "mixed") == b  # cached per shape class
    r = _eigen.eigsh_lm(op, 30, block=None)
    assert r.info["block"] == b and r.info["block_chosen"] and r.info["converged"]
    assert _eigen._BLOCK_SEEN[key][b] == r.info["vector_matvecs"]  # convergence history recorded
    ev_ref, U_ref = osp.eigen(*osp.operator(X), 30, 0)
    check_eigs(r.evals, r.evecs.cpu().numpy(), ev_ref, U_ref)
