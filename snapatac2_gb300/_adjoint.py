"""Gradient of the sum of the top-k eigenvalues with respect to the feature
weights, and a ``torch.autograd.Function`` around it.

The reference treats the feature weights as fixed inputs
(``snapatac2-python/src/embedding.rs:42-47``); this adds reverse-mode
differentiation through the whole operator set-up (row normalisation and the
degree normalisation, ``embedding.rs:139-152,315-326``) and the eigensolve
(Hellmann-Feynman: ∂f/∂A = U Uᵀ for the wanted eigenvectors U).  The chain
is in ``csrc/adjoint.cu``; it costs three FP64 SpMM passes.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _eigen, _lib
from ._binning import DeviceCSR


def _pad_block(b: int) -> int:
    for c in (4, 8, 16, 32):
        if b <= c:
            return c
    raise ValueError("k + 2 must be at most 32")


def eigsum_grad(op: _eigen.GramOperator, evals: np.ndarray, U: torch.Tensor) -> torch.Tensor:
    """∂(Σ evals)/∂w (FP64, length m) for eigenpairs (evals, U) of ``op``."""
    L = _lib.lib()
    dev = op.a.device
    n, m = op.n, op.m
    k = int(U.shape[1])
    B1 = _pad_block(k + 2)
    B2 = _pad_block(k + 1)
    sh = torch.cuda.current_stream(dev).cuda_stream
    f64 = dict(dtype=torch.float64, device=dev)
    U = U.to(dev, torch.float64).contiguous()
    lam = torch.as_tensor(np.asarray(evals, dtype=np.float64)).to(dev)
    ones_n, ones_m = torch.ones(n, **f64), torch.ones(m, **f64)
    in1, dbar = torch.empty(n, B1, **f64), torch.empty(n, **f64)
    zeh = torch.empty(m, B1, **f64)
    in2 = torch.empty(m, B2, **f64)
    P = torch.empty(n, B2, **f64)
    in3 = torch.empty(n, 4, **f64)
    g = torch.empty(m, 4, **f64)
    grad = torch.empty(m, **f64)
    cv = op.cvalues
    v = op.csr.data
    chk = _lib.check
    chk(L.sg_adjoint_stage1(n, k, U.data_ptr(), lam.data_ptr(), op.dinv.data_ptr(), op.rinv.data_ptr(), B1,
                            in1.data_ptr(), dbar.data_ptr(), sh), "adjoint stage 1")
    chk(L.sg_spmm(1, B1, m, op.colptr.data_ptr(), op.rowidx.data_ptr(), cv.data_ptr() if cv is not None else None,
                  in1.data_ptr(), zeh.data_ptr(), ones_m.data_ptr(), None, None, -1, sh), "adjoint Xᵀ pass")
    chk(L.sg_adjoint_stage2(m, k, zeh.data_ptr(), B1, op.w.data_ptr(), B2, in2.data_ptr(), sh), "adjoint stage 2")
    chk(L.sg_spmm(1, B2, n, op.csr.indptr.data_ptr(), op.csr.indices.data_ptr(), v.data_ptr() if v is not None else None,
                  in2.data_ptr(), P.data_ptr(), ones_n.data_ptr(), None, None, -1, sh), "adjoint X pass")
    chk(L.sg_adjoint_stage3(n, k, U.data_ptr(), op.dinv.data_ptr(), op.rinv.data_ptr(), dbar.data_ptr(),
                            P.data_ptr(), B2, in3.data_ptr(), sh), "adjoint stage 3")
    cv2 = None
    if cv is not None:
        cv2 = torch.empty_like(cv)
        chk(L.sg_square_values(cv.numel(), cv.data_ptr(), cv2.data_ptr(), sh), "square values")
    chk(L.sg_spmm(1, 4, m, op.colptr.data_ptr(), op.rowidx.data_ptr(), cv2.data_ptr() if cv2 is not None else None,
                  in3.data_ptr(), g.data_ptr(), ones_m.data_ptr(), None, None, -1, sh), "adjoint (X∘X)ᵀ pass")
    chk(L.sg_adjoint_final(m, k, op.w.data_ptr(), zeh.data_ptr(), B1, g.data_ptr(), grad.data_ptr(), sh),
        "adjoint final")
    return grad


class TopKEigenvalueSum(torch.autograd.Function):
    """f(w) = sum of the k largest-magnitude eigenvalues of the normalised
    cosine operator built from X with feature weights w; backward is the
    hand-written adjoint (``eigsum_grad``)."""

    @staticmethod
    def forward(ctx, w: torch.Tensor, csr: DeviceCSR, k: int, precision: str, block: int, solver_kw: dict):
        op = _eigen.build_operator(csr, w.detach().to(torch.float64).cpu().numpy())
        res = _eigen.eigsh_lm(op, k, precision=precision, block=block, **(solver_kw or {}))
        ctx.op, ctx.evals, ctx.U = op, res.evals, res.evecs
        return torch.tensor(float(np.sum(res.evals)), dtype=w.dtype, device=w.device)

    @staticmethod
    def backward(ctx, grad_out):
        g = eigsum_grad(ctx.op, ctx.evals, ctx.U)
        return (g * grad_out.to(g.dtype)).to(grad_out.dtype), None, None, None, None, None


def topk_eigenvalue_sum(w: torch.Tensor, X, k: int = 30, *, precision: str = "mixed", block: int = 8,
                        **solver_kw) -> torch.Tensor:
    """Differentiable sum of the top-``k`` (by magnitude) eigenvalues of the
    cosine operator of ``X`` (scipy CSR or DeviceCSR) with feature weights ``w``."""
    from .tools import csr_to_device
    dev = torch.device("cuda", torch.cuda.current_device())
    csr = csr_to_device(X, dev)
    return TopKEigenvalueSum.apply(w, csr, k, precision, block, solver_kw)
