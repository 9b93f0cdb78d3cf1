"""Thread count of the host BLAS that NumPy loaded (OpenBLAS builds only).

The batched eigensolver solves many small dense eigenproblems at once in a
thread pool; each LAPACK call there should run on one thread, or every pool
thread fans out to all cores and they contend.  OpenBLAS exports its own
setter; the shared library is found among the process's mapped files.
Anything else (another BLAS, no /proc) leaves the thread count unchanged.
"""
from __future__ import annotations

import contextlib
import ctypes

_PAIRS = (("scipy_openblas_get_num_threads64_", "scipy_openblas_set_num_threads64_"),
          ("scipy_openblas_get_num_threads", "scipy_openblas_set_num_threads"),
          ("openblas_get_num_threads64_", "openblas_set_num_threads64_"),
          ("openblas_get_num_threads", "openblas_set_num_threads"))
_found: list | None = None


def _controls() -> list:
    global _found
    if _found is None:
        _found = []
        try:
            with open("/proc/self/maps") as f:
                paths = sorted({ln.split()[-1] for ln in f if "openblas" in ln.lower() and ln.split()[-1].startswith("/")})
        except OSError:
            paths = []
        for p in paths:
            try:
                lib = ctypes.CDLL(p)
            except OSError:
                continue
            for get, put in _PAIRS:
                if hasattr(lib, get) and hasattr(lib, put):
                    g, s = getattr(lib, get), getattr(lib, put)
                    g.restype, g.argtypes = ctypes.c_int, []
                    s.restype, s.argtypes = None, [ctypes.c_int]
                    _found.append((g, s))
                    break
    return _found


@contextlib.contextmanager
def blas_threads(n: int):
    """Run the block with the host BLAS limited to n threads, then restore."""
    saved = []
    for g, s in _controls():
        saved.append((s, g()))
        s(n)
    try:
        yield
    finally:
        for s, v in saved:
            s(v)
