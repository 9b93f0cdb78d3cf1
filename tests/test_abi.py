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


def _declarations():
    """name -> (return type, [parameter types]) from the header."""
    src = open(os.path.join(ROOT, "include", "snapgb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    src = re.sub(r"#[^\n]*", "", src)
    out = {}
    for m in re.finditer(r"([\w\s\*]+?)\b(sg_\w+)\s*\(([^)]*)\)\s*;", src):
        ret = " ".join(m.group(1).split())
        params = [p.strip() for p in m.group(3).split(",")]
        if params == ["void"] or params == [""]:
            params = []
        types = [re.sub(r"\s*\b\w+$", "", p) if "*" not in p.split()[-1] else p for p in params]
        out[m.group(2)] = (ret, [" ".join(t.replace("*", " * ").split()) for t in types])
    return out


def _ctype_of(c_type: str):
    import ctypes
    if "*" in c_type:
        return ctypes.c_void_p, ctypes.c_char_p
    base = c_type.replace("const", "").strip()
    table = {"int": ctypes.c_int, "int64_t": ctypes.c_int64, "uint32_t": ctypes.c_uint32,
             "uint64_t": ctypes.c_uint64, "double": ctypes.c_double}
    return (table[base],)


def test_python_signatures_match_header_arguments():
    """Every ctypes binding has the header's argument count and compatible
    types (pointers as void* / char*, integers and doubles of the same width),
    and the same return type."""
    from snapatac2_gb300 import _lib
    decl = _declarations()
    assert set(decl) == set(declared_symbols())
    for name, (ret, params) in decl.items():
        res, args = _lib.SIGNATURES[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for i, (c, py) in enumerate(zip(params, args)):
            assert py in _ctype_of(c), (name, i, c, py)
        assert res in _ctype_of(ret.replace("const char *", "char *").replace("const char*", "char *")), (name, ret)
