"""Generate ``tests/golden/api_signatures.json``: the signatures of the
reference's Python entry points on the path, read from its source with
``ast`` (nothing is imported), so that the drop-in test can check names,
order, kinds and defaults without the reference present.

Run from the repository root:  python tests/golden/make_api_signatures.py
"""
from __future__ import annotations

import ast
import json
import os

# root of the SnapATAC2 source tree the fixtures are cut from: the first
# command-line argument, else $SNAPATAC2_REFERENCE
import sys  # noqa: E402
REFERENCE_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SNAPATAC2_REFERENCE", "")
if not REFERENCE_ROOT:
    sys.exit("usage: python " + os.path.basename(__file__) + " <SnapATAC2 source root> (or set SNAPATAC2_REFERENCE)")

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF = os.path.join(REFERENCE_ROOT, "snapatac2-python/python/snapatac2")
TARGETS = [("pp", "import_fragments", "preprocessing/_basic.py"),
           ("pp", "add_tile_matrix", "preprocessing/_basic.py"),
           ("pp", "make_peak_matrix", "preprocessing/_basic.py"),
           ("pp", "make_gene_matrix", "preprocessing/_basic.py"),
           ("pp", "select_features", "preprocessing/_basic.py"),
           ("pp", "knn", "preprocessing/_knn.py"),
           ("tl", "spectral", "tools/_embedding.py")]


def signature(path: str, name: str) -> dict:
    tree = ast.parse(open(path).read())
    fn = next(n for n in tree.body if isinstance(n, ast.FunctionDef) and n.name == name)
    a = fn.args
    pos = a.posonlyargs + a.args
    defaults = [None] * (len(pos) - len(a.defaults)) + list(a.defaults)
    params = [{"name": p.arg, "kind": "positional", "default": None if d is None else ast.unparse(d)}
              for p, d in zip(pos, defaults)]
    params += [{"name": p.arg, "kind": "keyword", "default": None if d is None else ast.unparse(d)}
               for p, d in zip(a.kwonlyargs, a.kw_defaults)]
    return {"line": fn.lineno, "params": params}


def main() -> None:
    out = []
    for ns, name, rel in TARGETS:
        sig = signature(os.path.join(REF, rel), name)
        out.append({"namespace": ns, "name": name, "file": f"snapatac2-python/python/snapatac2/{rel}", **sig})
    with open(os.path.join(ROOT, "tests", "golden", "api_signatures.json"), "w") as fh:
        json.dump(out, fh, indent=1)
        fh.write("\n")


if __name__ == "__main__":
    main()
