"""Generate ``tests/golden/embedding.npz``: outputs of the reference's own
Python for the spectral path, run on small seeded inputs:

* ``eigen``        the Python string embedded in ``spectral_mf``
                   (snapatac2-python/src/embedding.rs:158-171), on the
                   oracle's degree-scaled operator of a 300-cell synthetic
                   matrix (``synthetic.binary_csr``, seed 5);
* ``nystrom``      the Python string embedded in ``nystrom``
                   (embedding.rs:222-229), on a seeded landmark matrix, a
                   chunk of cells, eigenvectors and eigenvalues with a
                   negative entry (so some d <= 0 are replaced);
* ``orthogonalize`` (snapatac2-python/python/snapatac2/tools/_embedding.py:397-413)
                   on a seeded n x k matrix and eigenvalues;
* ``SpectralMatrixFree.fit`` (_embedding.py:434-465, the Python twin of the
                   Rust ``spectral_mf`` normalisation and degree of
                   embedding.rs:133-152, 315-326) with the class's ``_eigen``
                   (_embedding.py:475-481), on the 300-cell matrix (binary and
                   with counts) and seeded feature weights: the normalised,
                   degree-scaled matrix and 1/D handed to ``_eigen`` are
                   captured, and the eigenvalues kept.

The strings are cut out of the Rust source and the function out of the
Python source (``ast``), then executed with NumPy / SciPy only.  Inputs
are rebuilt by the test from the same seeds; only outputs are stored.

Run from the repository root:  python tests/golden/make_embedding_golden.py
"""
from __future__ import annotations

import ast
import os
import re
import sys

import numpy as np
import scipy.sparse as sp

# root of the SnapATAC2 source tree the fixtures are cut from: the first
# command-line argument, else $SNAPATAC2_REFERENCE
REFERENCE_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SNAPATAC2_REFERENCE", "")
if not REFERENCE_ROOT:
    sys.exit("usage: python " + os.path.basename(__file__) + " <SnapATAC2 source root> (or set SNAPATAC2_REFERENCE)")

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
REF_RS = os.path.join(REFERENCE_ROOT, "snapatac2-python/src/embedding.rs")
REF_PY = os.path.join(REFERENCE_ROOT, "snapatac2-python/python/snapatac2/tools/_embedding.py")


def embedded(name: str):
    src = open(REF_RS).read()
    m = re.search(r'"(def ' + name + r'\(.*?)",\n', src, re.S)
    ns: dict = {}
    exec(compile(m.group(1), REF_RS, "exec"), ns)
    return ns[name]


def python_function(name: str, ns: dict | None = None):
    fn = next(n for n in ast.parse(open(REF_PY).read()).body if isinstance(n, ast.FunctionDef) and n.name == name)
    ns = {"np": np} if ns is None else ns
    exec(compile(ast.Module(body=[fn], type_ignores=[]), REF_PY, "exec"), ns)
    return ns[name]


def python_class(name: str, ns: dict):
    cls = next(n for n in ast.parse(open(REF_PY).read()).body if isinstance(n, ast.ClassDef) and n.name == name)
    exec(compile(ast.Module(body=[cls], type_ignores=[]), REF_PY, "exec"), ns)
    return ns[name]


def spectral_mf_inputs(valued: bool):
    from snapatac2_gb300 import synthetic as S
    B = S.binary_csr(300, 2000, nnz_per_cell=60, seed=5)
    vals = np.random.default_rng(7).integers(1, 4, B.nnz).astype(np.float64) if valued else np.ones(B.nnz)
    X = sp.csr_matrix((vals, B.indices, B.indptr), shape=B.shape)
    w = np.random.default_rng(6).uniform(0.5, 3.0, B.shape[1])
    return X, w


def spectral_mf(X, w):
    import logging
    import scipy
    import scipy.sparse.linalg  # noqa: F401
    eig = python_function("_eigen", {"np": np, "sp": scipy})
    captured = {}

    def capture(Xs, dinv, k):
        captured["X"], captured["dinv"] = sp.csr_matrix(Xs), np.asarray(dinv)
        return eig(Xs, dinv, k)

    cls = python_class("SpectralMatrixFree", {"np": np, "sp": scipy, "_eigen": capture, "logging": logging})
    model = cls(out_dim=8, feature_weights=w).fit(X, verbose=0)
    Xs = captured["X"]
    Xs.sort_indices()
    return Xs, captured["dinv"], np.real(model.evals)


def eigen_inputs():
    from oracle import spectral as osp
    from snapatac2_gb300 import synthetic as S
    B = S.binary_csr(300, 2000, nnz_per_cell=60, seed=5)
    X = sp.csr_matrix((np.ones(B.nnz), B.indices, B.indptr), shape=B.shape)
    Xn = osp.normalize(X, osp.idf(X))
    Xs, dinv = osp.degree_scale(Xn)
    return Xs, dinv


def nystrom_inputs():
    rng = np.random.default_rng(9)
    seed = sp.random(120, 400, density=0.05, format="csr", random_state=1)
    sample = sp.random(250, 400, density=0.05, format="csr", random_state=2)
    evecs = rng.standard_normal((120, 6))
    evals = np.array([0.9, 0.6, 0.4, 0.3, 0.2, -0.35])
    return seed, sample, evecs, evals


def orthogonalize_inputs():
    rng = np.random.default_rng(4)
    q = rng.standard_normal((500, 7)) @ np.diag([3.0, 2.0, 1.5, 1.0, 0.7, 0.4, 0.2])
    evals = np.array([0.95, 0.8, 0.6, 0.5, 0.3, 0.25, 0.1])
    return evals, q


def main() -> None:
    out = {}
    Xs, dinv = eigen_inputs()
    ev, U = embedded("eigen")(Xs, dinv, 8, 0)
    out["eigen_evals"], out["eigen_evecs"] = ev, U
    seed, sample, evecs, evals = nystrom_inputs()
    out["nystrom_q"] = embedded("nystrom")(seed, sample, evecs.copy(), evals)
    evals, q = orthogonalize_inputs()
    e, V = python_function("orthogonalize")(evals, q)
    out["orth_evals"], out["orth_evecs"] = np.real(e), np.real(V)
    for tag, valued in (("mf", False), ("mfv", True)):
        X, w = spectral_mf_inputs(valued)
        Xs, dinv, ev = spectral_mf(X, w)
        out[f"{tag}_xs_data"], out[f"{tag}_xs_indices"], out[f"{tag}_xs_indptr"] = Xs.data, Xs.indices, Xs.indptr
        out[f"{tag}_dinv"], out[f"{tag}_evals"] = dinv, ev
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "embedding.npz"), **out)


if __name__ == "__main__":
    main()
