"""Build recipe of the CPU oracle (test infrastructure only).

Compiles ``oracle.cpp`` with the host C++ compiler into
``oracle/_build/liboracle.so``.  The reference (Particulator.jl) is Julia and
cannot be compiled or run here, so there is no ``oracle/_ref`` build: the
oracle is a restatement, parity unpinned.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "liboracle.so")


def build_oracle(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "oracle.cpp")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    # -ffp-contract=off keeps Float64 results independent of the host's FMA use
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", src, "-o", LIB_PATH]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stdout.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {r.stderr}")
    return LIB_PATH


if __name__ == "__main__":
    print(build_oracle(verbose=True, force="--force" in sys.argv))
