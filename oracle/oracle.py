"""ctypes front end of the CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``.  The product package never imports it.

The functions take numpy arrays in the layout of the reference API (sdf
``[X,Y,Z]``, deform ``[X,Y,Z,3]``) and compute in float64.  ``dtype`` names the
precision the reference would run in, which decides how ``isovalue`` and the
padding value ``isovalue + 1`` are rounded before they reach the kernels
(diso/__init__.py:52 pads with the Python float ``isovalue + 1``; src/pybind.cpp
passes ``isovalue`` as the extractor's scalar type).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
MC, DMC = 0, 1

_lock = threading.Lock()
_lib = None


class _Mesh(ctypes.Structure):
    _fields_ = [
        ("nv", ctypes.c_int64),
        ("nf", ctypes.c_int64),
        ("fw", ctypes.c_int),
        ("empty_guard", ctypes.c_int),
        ("verts", ctypes.POINTER(ctypes.c_double)),
        ("faces", ctypes.POINTER(ctypes.c_int64)),
        ("n_used", ctypes.c_int64),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    src = os.path.join(HERE, "oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    return LIB


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB)
            dp = ctypes.POINTER(ctypes.c_double)
            L.oracle_extract.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(_Mesh)]
            L.oracle_extract.restype = ctypes.c_int
            L.oracle_mesh_free.argtypes = [ctypes.POINTER(_Mesh)]
            L.oracle_backward.argtypes = [ctypes.c_int, dp, dp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_int, dp, ctypes.c_int64,
                                          dp, dp, ctypes.c_int]
            L.oracle_backward.restype = ctypes.c_int
            L.oracle_split_config.argtypes = [dp, ctypes.POINTER(ctypes.c_int64)]
            L.oracle_num_threads.restype = ctypes.c_int
            _lib = L
    return _lib


def iso_values(isovalue: float, dtype: str):
    """(iso, padval) exactly as the reference's kernels see them."""
    if dtype in ("float32", "f32"):
        return float(np.float32(isovalue)), float(np.float32(float(isovalue) + 1.0))
    return float(isovalue), float(isovalue) + 1.0


def _dp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _prep(sdf, deform):
    sdf = np.ascontiguousarray(sdf, dtype=np.float64)
    if deform is not None:
        deform = np.ascontiguousarray(deform, dtype=np.float64)
        assert deform.shape == sdf.shape + (3,)
    return sdf, deform


def extract(method: int, sdf, deform=None, isovalue: float = 0.0, normalize: bool = True,
            return_quads: bool = False, dtype: str = "float32"):
    """Forward of DiffMC (method=MC) or DiffDMC (method=DMC).

    Returns (verts [V,3] float64, faces [F,k] int64, info dict).  When the
    reference's empty-surface guard fires, faces has the reference's empty shape
    ([0,3] for MC, [0,4] for DMC) and info["empty_guard"] is True.
    """
    sdf, deform = _prep(sdf, deform)
    iso, pad = iso_values(isovalue, dtype)
    m = _Mesh()
    rc = lib().oracle_extract(method, _dp(sdf), _dp(deform), *sdf.shape, iso, pad, int(normalize),
                              int(return_quads), ctypes.byref(m))
    if rc != 0:
        raise RuntimeError(f"oracle_extract failed: {rc}")
    try:
        nv, nf, fw = m.nv, m.nf, m.fw
        if m.empty_guard:
            return (np.zeros((0, 3)), np.zeros((0, 4 if method == DMC else 3), np.int64),
                    {"empty_guard": True, "n_used": 0})
        verts = np.ctypeslib.as_array(m.verts, shape=(nv * 3,)).reshape(nv, 3).copy() if nv else np.zeros((0, 3))
        faces = (np.ctypeslib.as_array(m.faces, shape=(nf * fw,)).reshape(nf, fw).copy() if nf
                 else np.zeros((0, fw), np.int64))
        return verts, faces, {"empty_guard": False, "n_used": m.n_used}
    finally:
        lib().oracle_mesh_free(ctypes.byref(m))


def backward(method: int, sdf, deform, grad_verts, isovalue: float = 0.0, normalize: bool = True,
             dtype: str = "float32", exact: bool = False):
    """dL/dsdf and dL/ddeform (None without deform) for dL/dverts = grad_verts (final verts).

    exact=False reproduces the reference's DMC backward, in which every patch of a
    multi-patch cell receives the first patch's gradient (src/cudualmc.cu:990);
    exact=True gives the true derivative.  MC is the same either way."""
    sdf, deform = _prep(sdf, deform)
    iso, pad = iso_values(isovalue, dtype)
    gv = np.ascontiguousarray(grad_verts, dtype=np.float64).reshape(-1, 3)
    gs = np.zeros(sdf.shape, np.float64)
    gd = np.zeros(sdf.shape + (3,), np.float64) if deform is not None else None
    rc = lib().oracle_backward(method, _dp(sdf), _dp(deform), *sdf.shape, iso, pad, int(normalize),
                               _dp(gv), gv.shape[0], _dp(gs), _dp(gd), int(bool(exact)))
    if rc != 0:
        raise RuntimeError(f"oracle_backward failed: {rc} (grad_verts rows do not match the mesh)")
    return gs, gd


def split_config(verts, quad) -> int:
    """1 or 2: the triangle pair the reference's quad split picks (0 if NaN)."""
    v = np.ascontiguousarray(verts, dtype=np.float64)
    q = np.ascontiguousarray(quad, dtype=np.int64)
    return lib().oracle_split_config(_dp(v), q.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))


def num_threads() -> int:
    return lib().oracle_num_threads()
