"""The C-ABI library loads on a CPU-only host and exports every symbol that
include/snapgb300.h declares (no compute calls without a GPU)."""
import os
import re

from conftest import ROOT


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "snapgb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sg_\w+)\s*\(", src)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "sg_tile_plan" in syms and "sg_version" in syms


def test_library_exports_all_declared(built_lib):
    for s in declared_symbols():
        assert hasattr(built_lib, s), f"{s} declared in snapgb300.h but not exported"


def test_python_signatures_cover_header(built_lib):
    from snapatac2_gb300 import _lib
    missing = [s for s in declared_symbols() if s not in _lib.SIGNATURES]
    assert not missing, missing


def test_version_and_status(built_lib):
    assert built_lib.sg_version() >= 100
    assert built_lib.sg_status_string(2) == b"position out of range of the genome or chromosome"


def test_integration_guide_indexes_every_entry_point():
    """INTEGRATION.md's entry-point index names every declared function."""
    doc = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    missing = [s for s in declared_symbols() if f"`{s}`" not in doc]
    assert not missing, missing
