"""Build the CUDA library libvfs_poisson.so for sm_103a (in-tree, no cmake).

Translation units are compiled in parallel; setup.cu, noalloc.cu and ibm.cu
are compiled with -fmad=false (ibm.cu's host code also without contraction)
so that the grid, operator, right-hand-side, projection and classification
code rounds every operation in the reference's source order.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                 # vfs-wind_gb300/
REPO = os.path.dirname(ROOT)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
OUT_DIR = os.path.join(ROOT, "lib")
LIB = os.path.join(OUT_DIR, "libvfs_poisson.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
UNITS = {
    "setup.cu": ["-fmad=false"],
    "solve.cu": [],
    "poisson.cu": [],
    "noalloc.cu": ["-fmad=false"],
    "ibm.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"],
    "unet.cu": [],
    "io.cpp": ["-Xcompiler", "-ffp-contract=off"],
}


def _nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _sources():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)
            if f.endswith((".cu", ".cuh", ".h", ".cpp"))] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in _sources())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    nvcc = _nvcc()
    objs = []

    def compile_one(name):
        obj = os.path.join(OUT_DIR, os.path.splitext(name)[0] + ".o")
        cmd = [nvcc, *ARCH, *COMMON, *UNITS[name], "-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        return obj

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_one, UNITS))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
