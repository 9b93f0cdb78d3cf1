"""Compensated FP32 SpMM (sg_spmm_ds) of the eigensolver's correction sweep.

Checked against extended-precision NumPy sums (np.longdouble) on binary and
valued matrices with skewed row lengths and empty rows: every output within
(k + 8) 2^-46 of Σ|terms| for a row of k terms (FP64 recursive summation is
within k 2^-53), i.e. FP64-class; against the FP64 gather kernel to the same
bound; all four variants (index chunks in flight, static or counter-driven
rows) bitwise equal and repeatable; and sg_lanczos with the compensated sweep
against the FP64 sweep (eigenvalues 1e-12 relative, vectors 1e-9 rad).
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp


def _matrix(rows, cols, valued, seed):
    rng = np.random.default_rng(seed)
    lens = np.minimum((rng.pareto(1.2, rows) * 20).astype(np.int64), cols)
    lens[rng.random(rows) < 0.05] = 0
    indptr = np.concatenate([[0], np.cumsum(lens)])
    idx = np.concatenate([np.sort(rng.choice(cols, size=L, replace=False)) for L in lens] or [np.zeros(0, int)])
    vals = rng.integers(1, 5, size=idx.size).astype(np.float32) if valued else None
    return indptr.astype(np.int64), idx.astype(np.int32), vals


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda() if x is not None else None


def _run(L, pass_, rows, ip, ix, vl, pairs, scale, dshift=None, y=None, variant=0, order=None):
    import torch
    out = torch.empty(rows, 32, dtype=torch.float64, device="cuda")  # pairs: same bytes
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    npos = order.numel() if order is not None else rows
    rc = L.sg_spmm_ds(pass_, npos, p(ip), p(ix), p(vl), pairs.data_ptr(), out.data_ptr(), p(scale), p(dshift), p(y),
                      variant, p(order), cnt.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rc == 0
    return out


def _pairs_to_f64(out):
    f = out.view(dtype=__import__("torch").float32).cpu().numpy().reshape(out.shape[0], 32, 2).astype(np.float64)
    return f[..., 0] + f[..., 1]


@pytest.mark.gpu
@pytest.mark.parametrize("valued", [False, True])
def test_compensated_sums_are_fp64_class(valued):
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    rows, cols = 3000, 5000
    ip, ix, vl = _matrix(rows, cols, valued, 3 + valued)
    rng = np.random.default_rng(9)
    U = rng.standard_normal((cols, 32)) * np.exp(rng.uniform(-8, 8, (cols, 1)))  # magnitudes over 7 decades
    a = rng.uniform(0.5, 2.0, cols)
    scale = rng.uniform(0.1, 10.0, rows)
    d_ip, d_ix, d_vl = _dev(ip), _dev(ix), _dev(vl)
    d_U, d_a, d_s = _dev(U), _dev(a), _dev(scale)
    pairs = torch.empty(cols, 32, dtype=torch.float64, device="cuda")
    assert L.sg_ds_split(cols, d_a.data_ptr(), d_U.data_ptr(), pairs.data_ptr(), 0) == 0
    torch.cuda.synchronize()
    # the split is (hi, lo) with hi + lo = a*U to 2^-48
    v = a[:, None] * U
    assert np.all(np.abs(_pairs_to_f64(pairs) - v) <= 2.0 ** -47 * np.abs(v))
    X = sp.csr_matrix((vl if valued else np.ones(ix.size), ix, ip), shape=(rows, cols))
    Xl = X.astype(np.longdouble)
    exact = np.asarray(Xl @ v.astype(np.longdouble)) * scale[:, None].astype(np.longdouble)
    absum = np.asarray(abs(X) @ np.abs(v)) * scale[:, None]
    k = np.diff(ip)[:, None].astype(np.float64)
    tol = (k + 8) * 2.0 ** -46 * absum + 1e-300
    outs = [_run(L, 0, rows, d_ip, d_ix, d_vl, pairs, d_s, variant=vv) for vv in range(4)]
    got = _pairs_to_f64(outs[0])
    err = np.abs(got.astype(np.longdouble) - exact).astype(np.float64)
    assert np.all(err <= tol), float((err / np.maximum(absum, 1e-300)).max())
    for o in outs[1:]:  # every variant: same order of operations, same bits
        assert torch.equal(o, outs[0])
    # longest rows first (sg_row_order): same bits again
    npos = int(L.sg_row_order_positions(rows))
    order = torch.empty(npos, dtype=torch.int32, device="cuda")
    nb = int(L.sg_row_order_scratch_bytes(rows))
    scr = torch.empty(nb, dtype=torch.uint8, device="cuda")
    assert L.sg_row_order(rows, d_ip.data_ptr(), order.data_ptr(), scr.data_ptr(), nb, 0) == 0
    for vv in (2, 3):
        o = torch.empty_like(outs[0])
        cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert L.sg_spmm_ds(0, npos, d_ip.data_ptr(), d_ix.data_ptr(), d_vl.data_ptr() if d_vl is not None else None,
                            pairs.data_ptr(), o.data_ptr(), d_s.data_ptr(), None, None, vv, order.data_ptr(),
                            cnt.data_ptr(), 0) == 0
        torch.cuda.synchronize()
        assert torch.equal(o, outs[0])
    assert torch.equal(_run(L, 0, rows, d_ip, d_ix, d_vl, pairs, d_s, variant=3), outs[0])
    # pass 1 (FP64 out with the shift) against the FP64 gather kernel
    T = outs[0]
    Tv = _pairs_to_f64(T)
    n2 = 2000
    ip2, ix2, vl2 = _matrix(n2, rows, valued, 11)
    d_ip2, d_ix2, d_vl2 = _dev(ip2), _dev(ix2), _dev(vl2)
    y = rng.standard_normal((n2, 32))
    a2, dsh = rng.uniform(0.5, 2, n2), rng.uniform(0, 1, n2)
    d_y, d_a2, d_dsh = _dev(y), _dev(a2), _dev(dsh)
    W = _run(L, 1, n2, d_ip2, d_ix2, d_vl2, T, d_a2, d_dsh, d_y, variant=1).cpu().numpy()
    X2 = sp.csr_matrix((vl2 if valued else np.ones(ix2.size), ix2, ip2), shape=(n2, rows))
    ex2 = np.asarray(X2.astype(np.longdouble) @ Tv.astype(np.longdouble)) * a2[:, None] - dsh[:, None] * y
    abs2 = np.asarray(abs(X2) @ np.abs(Tv)) * a2[:, None] + np.abs(dsh[:, None] * y)
    k2 = np.diff(ip2)[:, None].astype(np.float64)
    err2 = np.abs(W.astype(np.longdouble) - ex2).astype(np.float64)
    assert np.all(err2 <= (k2 + 8) * 2.0 ** -46 * abs2 + 1e-300)
    # the FP64 kernel on the same operand agrees to the same bound
    Tf = _dev(Tv)
    W64 = torch.empty(n2, 32, dtype=torch.float64, device="cuda")
    p = lambda t: t.data_ptr() if t is not None else None  # noqa: E731
    assert L.sg_spmm(1, 32, n2, p(d_ip2), p(d_ix2), p(d_vl2), Tf.data_ptr(), W64.data_ptr(), d_a2.data_ptr(),
                     d_dsh.data_ptr(), d_y.data_ptr(), 0, 0) == 0
    torch.cuda.synchronize()
    assert np.all(np.abs(W64.cpu().numpy() - W) <= (k2 + 8) * 2.0 ** -46 * abs2 + 1e-300)


@pytest.mark.gpu
def test_spmm_ds_refuses_bad_arguments():
    import torch
    from snapatac2_gb300 import _lib
    L = _lib.lib()
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    ip = torch.zeros(2, dtype=torch.int64, device="cuda")
    p = buf.data_ptr()
    assert L.sg_spmm_ds(2, 1, ip.data_ptr(), p, None, p, p, p, None, None, 0, None, None, 0) == _lib.SG_ERR_ARG
    assert L.sg_spmm_ds(0, 1, ip.data_ptr(), p, None, p, p, p, p, p, 0, None, None, 0) == _lib.SG_ERR_ARG  # shift in pass 0
    assert L.sg_spmm_ds(0, 1, ip.data_ptr(), p, None, p, p, p, None, None, 2, None, None, 0) == _lib.SG_ERR_ARG  # no counter
    assert L.sg_spmm_ds(0, 1, ip.data_ptr(), p, None, p + 8, p, p, None, None, 0, None, None, 0) == _lib.SG_ERR_ARG  # misaligned
    assert L.sg_spmm_ds(0, 4, ip.data_ptr(), p, None, p, p, p, None, None, 1, ip.data_ptr(), None, 0) == _lib.SG_ERR_ARG  # order, static
    assert L.sg_spmm_ds_variants() == 4


@pytest.mark.gpu
def test_lanczos_compensated_sweep_matches_fp64_sweep():
    import torch
    from snapatac2_gb300 import _lib
    from test_lanczos_abi import _gram_op, _operator
    from test_spectral import check_eigs
    X, op = _operator(n=4000, m=60000, nnz=450, seed=17)
    L = _lib.lib()
    k, block = 30, 8
    gop = _gram_op(op)
    res = []
    for refine in (1, 2):
        opts = _lib.LanczosOpts()
        opts.refine = refine
        opts.max_restarts = -1
        opts.variant_t = opts.variant_x = opts.refine_variant_t = opts.refine_variant_x = -1
        nb = int(L.sg_lanczos_work_bytes(0, block, k, op.n, op.m, 0, 0))
        work = torch.empty(nb, dtype=torch.uint8, device="cuda")
        evals = np.empty(k)
        U = torch.empty(op.n, k, dtype=torch.float64, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        rc = L.sg_lanczos(ctypes.byref(gop), 0, block, k, 0, ctypes.byref(opts), work.data_ptr(), nb,
                          evals.ctypes.data, U.data_ptr(), None, None, st.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert rc == 0
        res.append((evals, U.cpu().numpy()))
    check_eigs(res[0][0], res[0][1], res[1][0], res[1][1], rtol=1e-12, angle=1e-9, positive_only=False)
