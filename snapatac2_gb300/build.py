"""In-tree build of ``libsnapgb300.so`` for sm_103a (nvcc, no cmake).

Each ``csrc/*.cu`` translation unit is compiled in parallel to an object in
``snapatac2_gb300/_build/`` and the objects are linked into
``snapatac2_gb300/libsnapgb300.so`` (static CUDA runtime).  Rebuilds only
what changed.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

_HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(_HERE, "csrc")
BUILD = os.path.join(_HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(_HERE), "include")
LIB = os.path.join(_HERE, "libsnapgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    n = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(n):
        raise RuntimeError("nvcc not found")
    return n


def _newest_dep() -> float:
    deps = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))
    return max((os.path.getmtime(d) for d in deps), default=0.0)


def build_library(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    hdr = _newest_dep()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    objs, procs = [], []
    for s in srcs:
        o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
        objs.append(o)
        if not force and os.path.exists(o) and os.path.getmtime(o) >= max(os.path.getmtime(s), hdr):
            continue
        cmd = [nvcc, *ARCH, *FLAGS, "-c", s, "-o", o + ".tmp"]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT), s, o))
    failed = []
    for p, s, o in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append(f"{s}:\n{out}")
        else:
            os.replace(o + ".tmp", o)
            if verbose and out.strip():
                print(out, file=sys.stderr)
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    if force or procs or not os.path.exists(LIB) or \
            os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
