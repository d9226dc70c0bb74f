"""Build libgbcodeml.so in-tree with nvcc for sm_103a (GB300).

    python -m cucodeml_gb300.build [--force]

Each translation unit is compiled in parallel into cucodeml_gb300/_build/,
then linked (static cudart) into cucodeml_gb300/libgbcodeml.so.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libgbcodeml.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["runtime.cu", "batch.cu", "k_fp64.cu", "adjoint.cu", "fast.cu", "k_fast.cu", "k_fast_bwd.cu", "k_umma.cu", "noalloc.cu", "beb.cu", "beb_clade.cu", "clade.cu", "se.cu", "model.cpp", "patterns.cpp", "ng86.cpp", "betaw.cpp"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA library cannot be built")
    return p


def _deps() -> list:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "gbcodeml.h")]


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3",
           "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cu"):
        cmd[1:1] = ["-Xptxas", "-v"] if os.environ.get("GB_PTXAS_VERBOSE") else []
    else:
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if os.environ.get("GB_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False) -> str:
    """Compile (if any source is newer than the library) and return the .so path."""
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in _deps()):
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
