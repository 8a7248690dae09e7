"""Builds libocean_gpu.so in-tree for sm_103a (GB300) with nvcc.

Each translation unit is compiled in parallel; the library is linked next to
this file.  No cmake, no torch extension machinery: the product is a plain
C-ABI shared library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libocean_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]

SOURCES = {
    "ocn_capi.cu": [],
    "ocn_kernels.cu": [],
    "ocn_cf.cu": ["-fmad=false"],
    "ocn_gmres.cu": [],
    "ocn_mixed.cu": [],
    "ocn_valence.cu": [],
    "ocn_setup.cpp": [],
    "ocn_io.cpp": [],
}


def nvcc() -> str:
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str], verbose: bool) -> str:
    obj = os.path.join(BUILD, src + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp, os.path.join(CSRC, "ocn_internal.h"), os.path.join(CSRC, "ocn_kmesh_dft.cuh"),
            os.path.join(ROOT, "include", "ocean_gpu.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", srcp, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + extra + ["-x", "c++", "-c", srcp, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    if force:
        for f in os.listdir(BUILD):
            os.remove(os.path.join(BUILD, f))
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), SOURCES.items()))
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
