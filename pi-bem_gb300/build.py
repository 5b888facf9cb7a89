"""Builds libpibem_gb300.so (CUDA for sm_103a + C++ host code) in-tree.

Usage: python pi-bem_gb300/build.py   (or through __graft_entry__.build()).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpibem_gb300.so")
SOURCES = ["setup.cu", "fmm.cu", "m2l_tc.cu", "ozaki_tc.cu", "levels.cu", "krylov.cu", "capi.cu", "projection.cu", "octree.cu", "tree.cpp",
           "prm.cpp", "mesh_io.cpp"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction: the quadrature
# points and the octree keys must round exactly as in the CPU oracle.
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
          "-Xcompiler", "-ffp-contract=off", "-lineinfo"]


def _compile(src: str) -> str:
    obj = os.path.join(OUT, src + ".o")
    path = os.path.join(CSRC, src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(
        os.path.getmtime(path), *(os.path.getmtime(os.path.join(CSRC, h)) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh")))
    ):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, *GENCODE, *COMMON, "-c", path, "-o", obj]
    else:
        cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off",
               "-I/usr/local/cuda/include", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        cmd = [NVCC, *GENCODE, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lcudart", "-lgomp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
