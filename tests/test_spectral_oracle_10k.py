"""Spectral embedding at 10,000 cells x 500,000 features (~4,000 nonzeros
per cell, the benchmark's generator) against the oracle's SciPy ARPACK
``eigsh`` -- the reference's own call (snapatac2-python/src/embedding.rs:
155-188) -- on the same matrix, for the mixed and the all-FP64 forms.

The oracle's matvec runs as the OpenMP restatement (``oracle/gram.c``); a
CPU test pins it to SciPy's single-threaded products on a smaller matrix.
Tolerances: eigenvalues within 1e-5 relative, principal angles within 1e-4
rad per cluster of eigenvalues closer than 1e-3 relative (``check_eigs``).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from oracle import spectral as osp
from snapatac2_gb300 import synthetic as syn
from test_spectral import check_eigs


# ----------------------------------------------------------------- CPU -----
def test_threaded_oracle_matvec_matches_scipy():
    B = syn.binary_csr(600, 40_000, nnz_per_cell=300, seed=3)
    X = sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)
    Xs, dinv = osp.operator(X)
    rng = np.random.default_rng(0)
    v = rng.standard_normal(X.shape[0])
    f = osp._threaded_matvec(Xs, dinv)
    want = Xs @ (v.T @ Xs).T - dinv * v
    assert np.allclose(f(v), want, rtol=1e-12, atol=1e-14)
    ev_a, U_a = osp.eigen(Xs, dinv, 20, 0)
    ev_b, U_b = osp.eigen(Xs, dinv, 20, 0, threaded=True)
    check_eigs(ev_b, U_b, ev_a, U_a, rtol=1e-10, angle=1e-8, positive_only=False)


# ----------------------------------------------------------------- GPU -----
@pytest.fixture(scope="module")
def c2_10k():
    import torch
    from snapatac2_gb300._binning import DeviceCSR
    dev = torch.device("cuda")
    n, m = 10_000, 500_000
    ip, ix, _ = syn.binary_csr_device(n, m, nnz_per_cell=4000, seed=4321, device=dev)
    X = sp.csr_matrix((np.ones(int(ix.numel())), ix.cpu().numpy(), ip.cpu().numpy()), shape=(n, m))
    ev_ref, U_ref = osp.eigen(*osp.operator(X), 30, 0, threaded=True)
    return DeviceCSR(ip, ix, None, (n, m)), ev_ref, U_ref


@pytest.mark.gpu
@pytest.mark.parametrize("precision,block", [("mixed", 8), ("fp64", 8), ("mixed", 32)])
def test_gpu_spectral_10k_against_arpack(c2_10k, precision, block):
    from snapatac2_gb300.tools import spectral_embedding
    csr, ev_ref, U_ref = c2_10k
    ev, U, info = spectral_embedding(csr, None, 30, 0, precision=precision, block=block, return_info=True)
    assert info["converged"], info
    check_eigs(ev, U.cpu().numpy(), ev_ref, U_ref)
