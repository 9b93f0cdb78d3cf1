"""Generate ``tests/golden/features.npz``: outputs of the reference's own
``_find_most_accessible_features``
(snapatac2-python/python/snapatac2/preprocessing/_basic.py:952-967) on
seeded count vectors with ties, zero counts and several quantiles/sizes.

The function is plain NumPy; its source is taken from the reference file
with ``ast`` and executed in a namespace holding only NumPy (the reference
package itself cannot be imported here: it needs its compiled extension).

Run from the repository root:  python tests/golden/make_feature_golden.py
"""
from __future__ import annotations

import ast
import os

import numpy as np

# root of the SnapATAC2 source tree the fixtures are cut from: the first
# command-line argument, else $SNAPATAC2_REFERENCE
import sys  # noqa: E402
REFERENCE_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SNAPATAC2_REFERENCE", "")
if not REFERENCE_ROOT:
    sys.exit("usage: python " + os.path.basename(__file__) + " <SnapATAC2 source root> (or set SNAPATAC2_REFERENCE)")

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.path.join(REFERENCE_ROOT, "snapatac2-python/python/snapatac2/preprocessing/_basic.py")
CASES = [  # (n features, fraction of zero counts, max count, lower, upper, total)
    (5000, 0.3, 5, 0.005, 0.005, 1000),
    (5000, 0.0, 50, 0.1, 0.0, 5000),
    (20000, 0.5, 3, 0.0, 0.2, 500),
    (20000, 0.05, 1000, 0.005, 0.005, 19000),
    (300, 0.9, 2, 0.05, 0.05, 10),
]


def reference_function():
    src = open(REF).read()
    fn = next(n for n in ast.parse(src).body
              if isinstance(n, ast.FunctionDef) and n.name == "_find_most_accessible_features")
    ns = {"np": np}
    exec(compile(ast.Module(body=[fn], type_ignores=[]), REF, "exec"), ns)
    return ns["_find_most_accessible_features"]


def main() -> None:
    f = reference_function()
    rng = np.random.default_rng(11)
    out = {}
    for i, (n, zf, mx, lo, up, tot) in enumerate(CASES):
        count = rng.integers(1, mx + 1, n).astype(np.float64)
        count[rng.random(n) < zf] = 0.0
        out[f"count{i}"] = count
        out[f"params{i}"] = np.array([lo, up, tot], dtype=np.float64)
        out[f"selected{i}"] = np.asarray(f(count, lo, up, tot), dtype=np.int64)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "features.npz"), **out)


if __name__ == "__main__":
    main()
