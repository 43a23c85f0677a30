"""In-tree build of libdiso_gb300.so for sm_103a (GB300) with nvcc."""
from __future__ import annotations

import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "libdiso_gb300.so")
SOURCES = [os.path.join(CSRC, "api.cu")]
DEPS = SOURCES + [os.path.join(CSRC, f) for f in ("backward.cuh", "common.cuh", "fields.cuh", "kernels.cuh", "mesh.cuh", "scan.cuh", "tma.cuh", "case_tables.h")] + [
    os.path.join(os.path.dirname(HERE), "include", "diso_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(home, "bin", "nvcc")


def needs_build() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(p) > t for p in DEPS if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not needs_build():
        return LIB
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-o", LIB + ".tmp", *SOURCES]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB
