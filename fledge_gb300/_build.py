"""Builds libflg.so (the CUDA kernels and the C ABI) in-tree for sm_103a.

Every translation unit is compiled by nvcc in parallel, then linked into
fledge_gb300/libflg.so with the CUDA runtime linked statically.  Objects go to
fledge_gb300/_build/.  A unit is recompiled when it or a header is newer than
its object.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libflg.so")

SOURCES = ["api.cu", "build.cu", "sort.cu", "collapse.cu", "trace.cu", "volume.cu",
           "adjoint.cu", "gen.cu", "pathtrace.cu", "ploc.cu", "sah.cu", "treelet.cu", "ply.cpp"]
HEADERS = [os.path.join(CSRC, "common.cuh"), os.path.join(CSRC, "internal.h"), os.path.join(CSRC, "volume.cuh"),
           os.path.join(ROOT, "include", "flg.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: no implicit multiply-add contraction, so the Morton, slab,
# Pluecker and tracking arithmetic rounds exactly as written.  Kernels that
# want FMA call fmaf() explicitly.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-fmad=false",
                     "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fvisibility=hidden,-ffp-contract=off",
                     "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    return "nvcc"


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + HEADERS)


def _compile(src: str, verbose: bool) -> str:
    s = os.path.join(CSRC, src)
    o = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    if _stale(o, s):
        cmd = [nvcc()] + NVCC_FLAGS + ["-c", s, "-o", o]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
    return o


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if force:
        for f in os.listdir(OUT):
            if f.endswith(".o"):
                os.remove(os.path.join(OUT, f))
    with ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + ".tmp"
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
