"""Drop-in check of the Python API (CPU): every parameter of the reference's
entry points on the path (``tests/golden/api_signatures.json``, read from the
reference source by ``tests/golden/make_api_signatures.py``) exists here with
the same name, position, kind and default."""
import ast
import inspect
import json
import os

import pytest

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "api_signatures.json")
with open(GOLDEN) as _fh:
    REFERENCE = json.load(_fh)


def _same_default(ref: str, ours) -> bool:
    want = ast.literal_eval(ref)
    if isinstance(want, list) and isinstance(ours, (list, tuple)):
        return list(ours) == want
    return type(ours) is type(want) and ours == want


@pytest.mark.parametrize("entry", REFERENCE, ids=[e["name"] for e in REFERENCE])
def test_signature_matches_reference(entry):
    import snapatac2_gb300 as snap
    fn = getattr(getattr(snap, entry["namespace"]), entry["name"])
    sig = inspect.signature(fn)
    where = f'{entry["file"]}:{entry["line"]}'
    positional = [p for p in sig.parameters.values()
                  if p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD)]
    ref_positional = [p for p in entry["params"] if p["kind"] == "positional"]
    assert [p.name for p in positional[:len(ref_positional)]] == [p["name"] for p in ref_positional], where
    for p in entry["params"]:
        assert p["name"] in sig.parameters, f'{where}: missing parameter {p["name"]}'
        ours = sig.parameters[p["name"]]
        if p["default"] is None:
            assert ours.default is inspect.Parameter.empty, f'{where}: {p["name"]} should be required'
        else:
            assert ours.default is not inspect.Parameter.empty, f'{where}: {p["name"]} needs a default'
            assert _same_default(p["default"], ours.default), \
                f'{where}: {p["name"]} default {ours.default!r}, reference {p["default"]}'
    # parameters added here come after the reference's and have defaults
    extra = [q for q in sig.parameters.values() if q.name not in {p["name"] for p in entry["params"]}
             and q.kind not in (q.VAR_POSITIONAL, q.VAR_KEYWORD)]
    assert all(q.default is not inspect.Parameter.empty for q in extra), where
