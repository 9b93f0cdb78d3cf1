"""Gradient of the top-k eigenvalue sum with respect to the feature weights.

Checked two ways, as the differentiation workload asks: against a dense FP64
reference gradient (torch autograd through the dense operator and eigvalsh,
on the CPU) and against central finite differences of the GPU forward along
random directions.  The sum is differentiable when |λ_k| > |λ_k+1|; the tests
pick k at a clear gap of the spectrum.
"""
import numpy as np
import pytest
import scipy.sparse as sp

from snapatac2_gb300 import synthetic as syn


def dense_topk_sum(w, Xd, k):
    """f(w) in dense FP64 torch (CPU), same chain as the GPU operator."""
    import torch
    n = Xd.shape[0]
    XW = Xd * w
    rho = XW.norm(dim=1)
    Xn = XW / rho[:, None]
    c = Xn.sum(0)
    d = Xn @ c
    s = (d - 1.0).rsqrt()
    K = Xn @ Xn.T
    A = s[:, None] * (K - torch.eye(n, dtype=Xd.dtype)) * s[None, :]
    lam = torch.linalg.eigvalsh(A)
    idx = torch.argsort(lam.abs(), descending=True)[:k]
    return lam[idx].sum(), lam


def pick_k(lam_sorted_abs, lo=6, hi=20):
    gaps = [(lam_sorted_abs[i - 1] - lam_sorted_abs[i]) / lam_sorted_abs[i - 1] for i in range(lo, hi)]
    return lo + int(np.argmax(gaps))


def small_problem(valued, n=300, m=2500, seed=5):
    B = syn.binary_csr(n, m, nnz_per_cell=120, n_clusters=4, enriched=500, seed=seed)
    data = np.ones(B.nnz)
    if valued:
        data = np.random.default_rng(seed).integers(1, 4, B.nnz).astype(float)
    X = sp.csr_matrix((data, B.indices, B.indptr), shape=B.shape)
    keep = np.asarray(X.sum(axis=0)).ravel() > 0
    X = sp.csr_matrix(X[:, keep])
    w = np.random.default_rng(seed + 1).uniform(0.5, 2.0, X.shape[1])
    return X, w


@pytest.mark.gpu
@pytest.mark.parametrize("valued", [False, True])
@pytest.mark.parametrize("precision,rtol", [("fp64", 1e-6), ("mixed", 1e-3)])
def test_gradient_matches_dense_fp64_reference(valued, precision, rtol):
    import torch
    from snapatac2_gb300._adjoint import topk_eigenvalue_sum
    X, w = small_problem(valued)
    Xd = torch.from_numpy(X.toarray())
    wt = torch.from_numpy(w).requires_grad_(True)
    _, lam = dense_topk_sum(wt.detach(), Xd, 40)
    k = pick_k(np.sort(np.abs(lam.numpy()))[::-1])
    f_ref, _ = dense_topk_sum(wt, Xd, k)
    (g_ref,) = torch.autograd.grad(f_ref, wt)
    wg = torch.from_numpy(w).cuda().requires_grad_(True)
    f = topk_eigenvalue_sum(wg, X, k, precision=precision, tol_vec=1e-12, tol_val=1e-12)
    f.backward()
    fr = float(f_ref.detach())
    assert abs(float(f.detach()) - fr) <= 1e-5 * abs(fr)
    g = wg.grad.cpu().numpy()
    err = np.abs(g - g_ref.numpy()).max() / np.abs(g_ref.numpy()).max()
    assert err <= rtol, err


@pytest.mark.gpu
def test_gradient_matches_dense_fp64_reference_2k_cells():
    """The dense FP64 reference gradient on a 2,000-cell subsample."""
    import torch
    from snapatac2_gb300._adjoint import topk_eigenvalue_sum
    X, w = small_problem(False, n=2000, m=6000, seed=13)
    Xd = torch.from_numpy(X.toarray())
    wt = torch.from_numpy(w).requires_grad_(True)
    _, lam = dense_topk_sum(wt.detach(), Xd, 40)
    k = pick_k(np.sort(np.abs(lam.numpy()))[::-1])
    f_ref, _ = dense_topk_sum(wt, Xd, k)
    (g_ref,) = torch.autograd.grad(f_ref, wt)
    wg = torch.from_numpy(w).cuda().requires_grad_(True)
    f = topk_eigenvalue_sum(wg, X, k, precision="fp64", tol_vec=1e-12, tol_val=1e-12)
    f.backward()
    assert abs(float(f.detach()) - float(f_ref.detach())) <= 1e-5 * abs(float(f_ref.detach()))
    g = wg.grad.cpu().numpy()
    assert np.abs(g - g_ref.numpy()).max() / np.abs(g_ref.numpy()).max() <= 1e-6


@pytest.mark.gpu
def test_gradient_matches_central_differences():
    import torch
    from snapatac2_gb300._adjoint import topk_eigenvalue_sum
    X, w = small_problem(False, n=1200, m=6000, seed=9)
    Xd = torch.from_numpy(X.toarray())
    _, lam = dense_topk_sum(torch.from_numpy(w), Xd, 40)
    k = pick_k(np.sort(np.abs(lam.numpy()))[::-1])
    kw = dict(precision="fp64", tol_vec=1e-13, tol_val=1e-13)
    wg = torch.from_numpy(w).cuda().requires_grad_(True)
    f = topk_eigenvalue_sum(wg, X, k, **kw)
    f.backward()
    g = wg.grad.cpu().numpy()
    rng = np.random.default_rng(0)
    eps = 1e-5
    for _ in range(64):  # 64 random unit directions
        v = rng.standard_normal(w.shape[0])
        v /= np.linalg.norm(v)
        fp = float(topk_eigenvalue_sum(torch.from_numpy(w + eps * v).cuda(), X, k, **kw))
        fm = float(topk_eigenvalue_sum(torch.from_numpy(w - eps * v).cuda(), X, k, **kw))
        fd = (fp - fm) / (2 * eps)
        an = float(g @ v)
        assert abs(fd - an) <= 1e-5 * max(abs(an), np.abs(g).max() * 1e-3), (fd, an)
