"""Build the in-tree shared library ``_build/libparticulator_gb300.so``.

Every translation unit is compiled for sm_103a only (``-gencode
arch=compute_103a,code=sm_103a``), in parallel, then linked with nvcc.  No
CMake, no torch extension machinery: the library is a plain C-ABI ``.so`` that
Julia (``ccall``), C/C++ and Python (``ctypes``) load alike.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_NAME = "libparticulator_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3"]
SOURCES = ["step.cu", "ctx.cu", "ctx_popops.cu", "ctx_hostio.cu", "ctx_learn.cu", "noalloc.cu", "mlp.cu", "learn.cu",
           "tables.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build particulator_gb300")


def _sources_newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build_library(verbose: bool = False, force: bool = False, ptxas_verbose: bool = False) -> str:
    """Compile and link the library; returns its path.  Raises on failure."""
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "particulator_gb300.h"))
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.rsplit(".", 1)[0] + ".o")
        objs.append(o)
        if force or _sources_newer(o, [s] + headers):
            cmd = [nvcc] + ARCH + NVCC_FLAGS
            if src.endswith(".cpp"):
                cmd += ["-x", "c++"]
            if ptxas_verbose and src.endswith(".cu"):
                cmd += ["-Xptxas", "-v"]
            cmd += ["-c", s, "-o", o]
            jobs.append(cmd)
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if verbose or ptxas_verbose or r.returncode != 0:
                sys.stdout.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"compilation failed: {' '.join(cmd)}\n{r.stderr}")
    if force or jobs or _sources_newer(LIB_PATH, objs):
        cmd = [nvcc] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stdout.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {r.stderr}")
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
