"""Compile the oracle's C restatements with gcc (ORACLE: test infrastructure)."""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
_SOURCES = {"tilebin": "tile_bin.c", "knn": "knn.c", "fragments": "fragments.c", "regions": "regions.c",
            "gram": "gram.c"}
_LOCK = threading.Lock()
_LIBS: dict[str, ctypes.CDLL] = {}


def _so_path(name: str) -> str:
    return os.path.join(_HERE, f"lib{name}_oracle.so")


def build_oracle(force: bool = False) -> None:
    """Compile every oracle C file into ``oracle/lib*_oracle.so``."""
    procs = []
    for name, src in _SOURCES.items():
        so = _so_path(name)
        s = os.path.join(_HERE, src)
        if not force and os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(s):
            continue
        tmp = so + f".tmp{os.getpid()}"
        procs.append((subprocess.Popen(
            ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-shared", "-fPIC", s, "-o", tmp, "-lm"]), tmp, so))
    for p, tmp, so in procs:
        if p.wait() != 0:
            raise RuntimeError(f"oracle build failed for {so}")
        os.replace(tmp, so)


def load_lib(name: str) -> ctypes.CDLL:
    with _LOCK:
        if name not in _LIBS:
            build_oracle()
            _LIBS[name] = ctypes.CDLL(_so_path(name))
        return _LIBS[name]
