"""ctypes binding of the C ABI in include/diso_gb300.h (libdiso_gb300.so).

The library is built in-tree by ``diso_gb300.build.build()`` (called from
``__graft_entry__.build()``).  There is no fallback: if the library is missing
or fails to load, every extraction raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdiso_gb300.so")

MC, DMC = 0, 1
F32, F64 = 0, 1
GRAD_EXACT = 1
GRAD_ZEROED = 2

# launch parameters of diso_tune_set
TUNE_PARAMS = {"count_ctas": 0, "emit_ctas": 1, "gather_ctas": 2, "fused_ctas": 3, "zero_ctas": 4, "edge_ctas": 5,
               "batch_ctas": 6, "zero_share": 7}

_lock = threading.Lock()
_lib = None


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 32), ("launches", ctypes.c_int64), ("total_ms", ctypes.c_double)]


class Counts(ctypes.Structure):
    _fields_ = [
        ("n_verts", ctypes.c_int64),
        ("n_faces", ctypes.c_int64),
        ("sdf_min", ctypes.c_double),
        ("sdf_max", ctypes.c_double),
        ("empty", ctypes.c_int32),
        ("emitted", ctypes.c_int32),
        ("n_active_tiles", ctypes.c_int64),
    ]


class SphereFieldDesc(ctypes.Structure):
    """diso_sphere_field: spheres [count][4] (x, y, z, r) in device memory, grid bounds, deform or NULL."""
    _fields_ = [
        ("spheres", ctypes.c_void_p),
        ("count", ctypes.c_int),
        ("lo", ctypes.c_double * 3),
        ("hi", ctypes.c_double * 3),
        ("deform", ctypes.c_void_p),
    ]


BRICK = 8
BRICK_OUTSIDE, BRICK_INSIDE = -1, -2


class BrickGridDesc(ctypes.Structure):
    """diso_brick_grid: dims, index [ceil(n/8)]^3 int32, values [count][8][8][8], deform or NULL, background."""
    _fields_ = [
        ("dims", ctypes.c_int * 3),
        ("index", ctypes.c_void_p),
        ("count", ctypes.c_int),
        ("values", ctypes.c_void_p),
        ("deform", ctypes.c_void_p),
        ("background", ctypes.c_double),
    ]


EXPORTS = {
    # name: (restype, argtypes)
    "diso_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "diso_destroy": (None, [ctypes.c_void_p]),
    "diso_segment_slots": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "diso_forward_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.POINTER(Counts)]),
    "diso_forward_emit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_void_p]),
    "diso_edge_record_slots": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int, ctypes.c_int64, ctypes.c_int64]),
    "diso_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_int,
                                    ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                    ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Counts)]),
    "diso_split_quads": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                        ctypes.c_void_p, ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p]),
    "diso_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p, ctypes.c_void_p]),
    "diso_backward_recompute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                               ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                               ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_isovalue_grad": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_forward_count_static": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int,
                                                 ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                 ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Counts)]),
    "diso_zero_grads": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_zero_count_share": (ctypes.c_double, []),
    "diso_forward_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SphereFieldDesc), ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.POINTER(Counts)]),
    "diso_backward_field": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SphereFieldDesc), ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_field_materialize": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(SphereFieldDesc), ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_forward_bricks": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BrickGridDesc), ctypes.c_double,
                                           ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                           ctypes.POINTER(Counts)]),
    "diso_backward_bricks": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(BrickGridDesc), ctypes.c_double,
                                            ctypes.c_double, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_bricks_materialize": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(BrickGridDesc), ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p]),
    "diso_mesh_normals": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_mesh_weld": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                      ctypes.c_void_p]),
    "diso_mesh_obj": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.POINTER(ctypes.c_int64), ctypes.c_void_p]),
    "diso_mesh_ply_bytes": (ctypes.c_int64, [ctypes.c_int, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]),
    "diso_mesh_ply": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_int64, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_timing": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "diso_timing_read": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int)]),
    "diso_tune_set": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]),
    "diso_tune_value": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "diso_scan_wait_probe": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint, ctypes.c_void_p]),
    "diso_scratch_bytes": (ctypes.c_int64, [ctypes.c_void_p]),
    "diso_last_error": (ctypes.c_char_p, []),
    "diso_version": (ctypes.c_char_p, []),
}


def lib():
    """The loaded library; raises RuntimeError when it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(
                    f"diso_gb300: CUDA library {LIB_PATH} is missing; build it with "
                    "`python -c 'import __graft_entry__ as g; g.build()'`")
            L = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in EXPORTS.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
    return _lib


def check(rc: int, what: str):
    if rc != 0:
        msg = lib().diso_last_error().decode(errors="replace")
        raise RuntimeError(f"diso_gb300 {what} failed (status {rc}): {msg}")


def dtype_tag(dtype: torch.dtype) -> int:
    if dtype == torch.float32:
        return F32
    if dtype == torch.float64:
        return F64
    raise ValueError(f"diso_gb300 supports float32 and float64, got {dtype}")


def iso_values(isovalue: float, dtype: torch.dtype):
    """(iso, padval) as the reference's kernels see them: the isovalue in the
    grid's dtype and the pad value isovalue + 1 computed in Python and then
    rounded to that dtype (diso/__init__.py:52)."""
    iso = float(isovalue.detach()) if isinstance(isovalue, torch.Tensor) else float(isovalue)
    if dtype == torch.float32:
        return float(np.float32(iso)), float(np.float32(iso + 1.0))
    return iso, iso + 1.0


def ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_of(device) -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class Extractor:
    """Owner of one native extractor (method x dtype) and its scratch."""

    def __init__(self, method: int, dtype: torch.dtype):
        self.method = method
        self.dtype = dtype
        # output capacities per grid shape from the last extraction of that shape
        # (dense grids and evaluated fields), for the single-call forward
        self.size_hints = {}
        self.field_hints = {}
        self.brick_hints = {}
        self._h = ctypes.c_void_p()
        check(lib().diso_create(method, dtype_tag(dtype), ctypes.byref(self._h)), "create")

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().diso_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def segment_slots(shape) -> int:
        return int(lib().diso_segment_slots(*shape))

    def count(self, sdf, iso, pad, seg) -> Counts:
        c = Counts()
        check(lib().diso_forward_count(self._h, ptr(sdf), *sdf.shape, iso, pad, ptr(seg),
                                       stream_of(sdf.device), ctypes.byref(c)), "forward count")
        return c

    def set_launch(self, params: dict):
        """Launch widths for this extractor's later calls ({name: value}, names of
        TUNE_PARAMS; 0 restores a default); outputs do not depend on them."""
        for name, value in params.items():
            check(lib().diso_tune_set(self._h, TUNE_PARAMS[name], int(value)), f"launch parameter {name}")

    def launch(self) -> dict:
        """The launch widths set on this extractor (0: default)."""
        return {name: int(lib().diso_tune_value(self._h, i)) for name, i in TUNE_PARAMS.items()}

    def scratch_bytes(self) -> int:
        """Device bytes held by this extractor's own scratch buffers."""
        return int(lib().diso_scratch_bytes(self._h))

    def timing(self, enable: bool):
        """Time every kernel this extractor launches (CUDA events on each launch's stream)."""
        check(lib().diso_timing(self._h, int(bool(enable))), "timing")

    def timing_read(self) -> dict:
        """{kernel: (launches, total ms)} of the launches since the last read."""
        arr = (KernelTime * 16)()
        n = ctypes.c_int(0)
        check(lib().diso_timing_read(self._h, arr, 16, ctypes.byref(n)), "timing read")
        return {arr[i].name.decode(): (int(arr[i].launches), float(arr[i].total_ms)) for i in range(n.value)}

    def record_slots(self, counts=None, n_verts=None, n_faces=None) -> int:
        """int64 slots of the edge record of a forward with these counts."""
        nv = int(counts.n_verts) if counts is not None else int(n_verts)
        nf = int(counts.n_faces) if counts is not None else int(n_faces)
        return int(lib().diso_edge_record_slots(self.method, dtype_tag(self.dtype), nv, nf))

    def forward(self, sdf, deform, iso, pad, seg, normalize, verts, faces, record) -> Counts:
        """Count, scan and emit into outputs of the given capacities in one call;
        Counts.emitted says whether they fitted (see diso_forward)."""
        c = Counts()
        check(lib().diso_forward(self._h, ptr(sdf), ptr(deform), *sdf.shape, iso, pad, ptr(seg), int(bool(normalize)),
                                 ptr(verts), verts.shape[0], ptr(faces), faces.shape[0], ptr(record),
                                 stream_of(sdf.device), ctypes.byref(c)), "forward")
        return c

    def emit(self, sdf, deform, iso, pad, seg, normalize, verts, faces, record=None):
        check(lib().diso_forward_emit(self._h, ptr(sdf), ptr(deform), *sdf.shape, iso, pad, ptr(seg),
                                      int(bool(normalize)), ptr(verts), ptr(faces), ptr(record),
                                      stream_of(sdf.device)),
              "forward emit")

    def split(self, verts, quads, tris) -> int:
        n = ctypes.c_int64(0)
        check(lib().diso_split_quads(self._h, ptr(verts), ptr(quads), quads.shape[0], ptr(tris), ctypes.byref(n),
                                     stream_of(verts.device)), "quad split")
        return int(n.value)

    def zero_grads(self, grad_sdf, grad_deform):
        """Zero the gradient buffers on a second stream of this extractor, beside the
        forward's kernels (see diso_zero_grads); the buffers are recorded on that
        stream, so torch does not reuse their memory before the zeros land."""
        dev = grad_sdf.device
        side = getattr(self, "_side", None)
        if side is None or side.device != dev:
            side = self._side = torch.cuda.Stream(dev)
        nb = lambda t: 0 if t is None else t.numel() * t.element_size()
        check(lib().diso_zero_grads(self._h, ptr(grad_sdf), nb(grad_sdf), ptr(grad_deform), nb(grad_deform),
                                    stream_of(dev), ctypes.c_void_p(side.cuda_stream)), "zero grads")
        grad_sdf.record_stream(side)
        if grad_deform is not None:
            grad_deform.record_stream(side)

    def forward_field(self, desc, shape, iso, pad, seg, normalize, verts, faces) -> Counts:
        """The forward of an evaluated field in one call (see diso_forward_field)."""
        c = Counts()
        check(lib().diso_forward_field(self._h, ctypes.byref(desc), *shape, iso, pad, ptr(seg), int(bool(normalize)),
                                       ptr(verts), verts.shape[0], ptr(faces), faces.shape[0], stream_of(verts.device),
                                       ctypes.byref(c)), "forward of a field")
        return c

    def backward_field(self, desc, shape, iso, pad, seg, normalize, grad_verts, grad_spheres, grad_deform,
                       exact=False):
        """Sphere-parameter (and deform) gradients of a forward_field (see diso_backward_field)."""
        check(lib().diso_backward_field(self._h, ctypes.byref(desc), *shape, iso, pad, ptr(seg), int(bool(normalize)),
                                        GRAD_EXACT if exact else 0, ptr(grad_verts), ptr(grad_spheres),
                                        ptr(grad_deform), stream_of(grad_verts.device)), "backward of a field")

    def forward_bricks(self, desc, iso, pad, seg, normalize, verts, faces) -> Counts:
        """The forward of a narrow band in one call (see diso_forward_bricks)."""
        c = Counts()
        check(lib().diso_forward_bricks(self._h, ctypes.byref(desc), iso, pad, ptr(seg), int(bool(normalize)),
                                        ptr(verts), verts.shape[0], ptr(faces), faces.shape[0],
                                        stream_of(verts.device), ctypes.byref(c)), "forward of a narrow band")
        return c

    def backward_bricks(self, desc, iso, pad, seg, normalize, grad_verts, grad_values, grad_deform, exact=False):
        """Gradients of a narrow band's slots (see diso_backward_bricks)."""
        check(lib().diso_backward_bricks(self._h, ctypes.byref(desc), iso, pad, ptr(seg), int(bool(normalize)),
                                         GRAD_EXACT if exact else 0, ptr(grad_verts), ptr(grad_values),
                                         ptr(grad_deform), stream_of(grad_verts.device)), "backward of a narrow band")

    # mesh consumers (diso_mesh_*): the extractor supplies the dtype and the scratch
    def mesh_normals(self, verts, faces, out):
        check(lib().diso_mesh_normals(self._h, ptr(verts), verts.shape[0], ptr(faces), faces.shape[0], faces.shape[1],
                                      ptr(out), stream_of(verts.device)), "vertex normals")

    def mesh_weld(self, verts, faces, tol, out_verts, out_faces):
        nv, nf = ctypes.c_int64(0), ctypes.c_int64(0)
        check(lib().diso_mesh_weld(self._h, ptr(verts), verts.shape[0], ptr(faces), faces.shape[0], faces.shape[1],
                                   float(tol), ptr(out_verts), ptr(out_faces), ctypes.byref(nv), ctypes.byref(nf),
                                   stream_of(verts.device)), "weld")
        return int(nv.value), int(nf.value)

    def mesh_obj(self, verts, normals, faces, text=None):
        n = ctypes.c_int64(0)
        check(lib().diso_mesh_obj(self._h, ptr(verts), ptr(normals), verts.shape[0], ptr(faces), faces.shape[0],
                                  faces.shape[1], ptr(text), text.numel() if text is not None else 0,
                                  ctypes.byref(n), stream_of(verts.device)), "OBJ text")
        return int(n.value)

    def mesh_ply(self, verts, normals, faces, body):
        check(lib().diso_mesh_ply(self._h, ptr(verts), ptr(normals), verts.shape[0], ptr(faces), faces.shape[0],
                                  faces.shape[1], ptr(body), stream_of(verts.device)), "PLY body")

    def backward(self, sdf, deform, iso, pad, seg, record, normalize, grad_verts, grad_sdf, grad_deform,
                 exact=False, zeroed=False):
        flags = (GRAD_EXACT if exact else 0) | (GRAD_ZEROED if zeroed else 0)
        check(lib().diso_backward(self._h, ptr(sdf), ptr(deform), *sdf.shape, iso, pad, ptr(seg), ptr(record),
                                  int(bool(normalize)), flags, ptr(grad_verts), ptr(grad_sdf),
                                  ptr(grad_deform), stream_of(sdf.device)), "backward")

    def backward_recompute(self, sdf, deform, iso, pad, seg, normalize, grad_verts, grad_sdf, grad_deform,
                           exact=False):
        """Backward of a forward that kept only its segment record: every element of
        grad_sdf (and grad_deform) is written (see diso_backward_recompute); the
        zeros that the extractor's second stream writes are joined into the caller's
        stream before the call returns its work to it."""
        flags = GRAD_EXACT if exact else 0
        check(lib().diso_backward_recompute(self._h, ptr(sdf), ptr(deform), *sdf.shape, iso, pad, ptr(seg),
                                            int(bool(normalize)), flags, ptr(grad_verts), ptr(grad_sdf),
                                            ptr(grad_deform), stream_of(sdf.device)), "backward (recompute)")

    def isovalue_grad(self, grad_sdf, seg=None):
        """dL/d(isovalue) = -(sum of dL/dsdf), as a 0-dim float64 tensor on the
        gradient's device (diso_isovalue_grad); `seg`, the forward's record, limits
        the reads to the point tiles near the surface."""
        out = torch.empty((), dtype=torch.float64, device=grad_sdf.device)
        check(lib().diso_isovalue_grad(self._h, ptr(grad_sdf), *grad_sdf.shape, ptr(seg), ptr(out),
                                       stream_of(grad_sdf.device)), "isovalue gradient")
        return out
