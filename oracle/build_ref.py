"""Build the reference's own CUDA extension (diso._C) from its unmodified sources.

TEST INFRASTRUCTURE ONLY.  This is the recipe for ``oracle/_ref/``: it compiles
``src/cumc.cu``, ``src/cudualmc.cu`` and ``src/pybind.cpp`` of a reference
checkout with direct nvcc/g++ commands against the installed torch headers
(one ``-gencode`` for sm_103a, ``-O3`` as the reference's setup.py uses),
without running the reference's own setup.py.  Output goes to ``oracle/_ref/`` only.

The reference extension runs only on a GPU, so it is used to produce the golden
fixtures under tests/golden/ (see tests/golden/make_golden.py); nothing in the
GPU tests, smoke() or bench.py loads it.

Usage:  python oracle/build_ref.py --src <reference checkout>
(default: the checkout named by the environment variable DISO_REFERENCE_SRC)
"""
from __future__ import annotations

import argparse
import importlib.util
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
DEFAULT_SRC = os.environ.get("DISO_REFERENCE_SRC")


def _torch_flags():
    import sysconfig

    import torch
    from torch.utils import cpp_extension as ce

    inc = [os.path.join(os.path.dirname(torch.__file__), "include"),
           os.path.join(os.path.dirname(torch.__file__), "include", "torch", "csrc", "api", "include"),
           sysconfig.get_paths()["include"]]
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    defs = ["-DTORCH_EXTENSION_NAME=_C", "-DTORCH_API_INCLUDE_EXTENSION_H", f"-D_GLIBCXX_USE_CXX11_ABI={abi}"]
    libdirs = ce.library_paths()
    return inc, defs, libdirs


def build(src: str = DEFAULT_SRC, verbose: bool = False):
    """Compile the three reference sources into oracle/_ref/_C.so and import it."""
    import subprocess

    if not src:
        raise RuntimeError("no reference checkout given (pass src or set DISO_REFERENCE_SRC)")
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "_C.so")
    srcs = [os.path.join(src, "src", f) for f in ("pybind.cpp", "cumc.cu", "cudualmc.cu")]
    if not os.path.exists(so) or any(os.path.getmtime(s) > os.path.getmtime(so) for s in srcs):
        inc, defs, libdirs = _torch_flags()
        incf = [f"-I{d}" for d in inc + [os.path.join(src, "src")]]
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        objs = []
        for s in srcs:
            o = os.path.join(OUT, os.path.basename(s) + ".o")
            if s.endswith(".cu"):
                cmd = [os.path.join(cuda, "bin", "nvcc"), "-O3", "-std=c++17",
                       "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler", "-fPIC",
                       "--expt-relaxed-constexpr", "-c", s, "-o", o] + incf + defs
            else:
                cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-c", s, "-o", o,
                       f"-I{cuda}/include"] + incf + defs
            if verbose:
                print(" ".join(cmd), flush=True)
            subprocess.run(cmd, check=True)
            objs.append(o)
        link = ["g++", "-shared", "-o", so] + objs + [f"-L{d}" for d in libdirs] + [
            f"-Wl,-rpath,{d}" for d in libdirs] + [f"-L{cuda}/lib64", "-lc10", "-lc10_cuda", "-ltorch",
                                                    "-ltorch_cpu", "-ltorch_cuda", "-ltorch_python", "-lcudart"]
        if verbose:
            print(" ".join(link), flush=True)
        subprocess.run(link, check=True)
    spec = importlib.util.spec_from_file_location("_C", so)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_reference(src: str = DEFAULT_SRC):
    """Import the reference's ``diso`` package (its own __init__.py) on top of the
    extension built by :func:`build`."""
    ext = build(src)
    sys.modules["diso_ref._C"] = ext
    spec = importlib.util.spec_from_file_location(
        "diso_ref", os.path.join(src, "diso", "__init__.py"), submodule_search_locations=[OUT])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["diso_ref"] = mod
    spec.loader.exec_module(mod)
    return mod


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=DEFAULT_SRC, required=DEFAULT_SRC is None)
    args = ap.parse_args()
    m = build(args.src, verbose=True)
    print("built", m.__file__, [n for n in dir(m) if n.startswith("CU")])
