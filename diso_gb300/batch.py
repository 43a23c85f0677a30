"""Batched extraction: many grids of uneven size, one launch per phase.

The reference has no batched call; its README runs a Python loop over one
extractor (README.md:61-70).  Here every phase (count, scan, emit, backward) of
all grids of a batch is one persistent launch over a flattened queue of their
tiles, with per-grid segments inside one scan:

* :func:`extract_batch` / :class:`DiffMCBatch` / :class:`DiffDMCBatch`: autograd,
  list of grids in, list of ``(verts, faces)`` out, each exactly what the
  single-grid module returns for that grid;
* :class:`BatchPlan`: fixed device buffers for a fixed list of grid shapes, the
  whole forward + backward captured once in a CUDA graph and replayed while the
  grids' contents change in place (capacity-bounded outputs; an overflow is
  reported and the plan can be re-sized).
"""
from __future__ import annotations

import ctypes

import torch
from torch import nn
from torch.autograd import Function

from . import _native as N


class Grid(ctypes.Structure):
    _fields_ = [
        ("sdf", ctypes.c_void_p),
        ("deform", ctypes.c_void_p),
        ("grad_sdf", ctypes.c_void_p),
        ("grad_deform", ctypes.c_void_p),
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("nz", ctypes.c_int),
        ("pad_", ctypes.c_int),
        ("isovalue", ctypes.c_double),
        ("padval", ctypes.c_double),
    ]


_BATCH_EXPORTS = {
    "diso_batch_record_slots": (ctypes.c_int64, [ctypes.POINTER(Grid), ctypes.c_int]),
    "diso_batch_prepare": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Grid), ctypes.c_int, ctypes.c_void_p,
                                          ctypes.c_void_p]),
    "diso_batch_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "diso_batch_results": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(N.Counts), ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int),
                                          ctypes.c_void_p]),
    "diso_batch_emit": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int64,
                                       ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]),
    "diso_batch_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p]),
}
N.EXPORTS.update(_BATCH_EXPORTS)


def _lib():
    L = N.lib()
    if not getattr(L, "_diso_batch_bound", False):
        for name, (res, args) in _BATCH_EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        L._diso_batch_bound = True
    return L


def _grids(sdfs, deforms, isos, dtype, grad_sdfs=None, grad_deforms=None):
    arr = (Grid * len(sdfs))()
    for i, s in enumerate(sdfs):
        iso, pad = N.iso_values(isos[i], dtype)
        d = deforms[i] if deforms is not None else None
        arr[i].sdf = s.data_ptr()
        arr[i].deform = d.data_ptr() if d is not None else None
        arr[i].grad_sdf = grad_sdfs[i].data_ptr() if grad_sdfs is not None else None
        arr[i].grad_deform = grad_deforms[i].data_ptr() if (grad_deforms is not None and d is not None) else None
        arr[i].nx, arr[i].ny, arr[i].nz = s.shape
        arr[i].isovalue, arr[i].padval = iso, pad
    return arr


class BatchResults:
    """Per-grid sizes and offsets of the last batched count."""

    def __init__(self, n):
        self.counts = (N.Counts * n)()
        self.voff = (ctypes.c_int64 * n)()
        self.foff = (ctypes.c_int64 * n)()
        self.overflow = ctypes.c_int(0)


class _Batch:
    """The native side of one batched extraction (an extractor + its batch state)."""

    def __init__(self, method, dtype):
        self.ex = N.Extractor(method, dtype)
        self.method, self.dtype = method, dtype

    def prepare(self, grids, record, device):
        N.check(_lib().diso_batch_prepare(self.ex._h, grids, len(grids), N.ptr(record), N.stream_of(device)),
                "batch prepare")

    def count(self, device):
        N.check(_lib().diso_batch_count(self.ex._h, N.stream_of(device)), "batch count")

    def results(self, n, device):
        r = BatchResults(n)
        N.check(_lib().diso_batch_results(self.ex._h, r.counts, r.voff, r.foff, ctypes.byref(r.overflow),
                                          N.stream_of(device)), "batch results")
        return r

    def edge_record(self, vcap, fcap, device):
        """A batch edge record for outputs of these capacities (int64, at least one slot)."""
        n = int(N.lib().diso_edge_record_slots(self.method, N.dtype_tag(self.dtype), int(vcap), int(fcap)))
        return torch.empty(max(1, n), dtype=torch.int64, device=device)

    def emit(self, normalize, verts, faces, device, record=None):
        N.check(_lib().diso_batch_emit(self.ex._h, int(bool(normalize)), N.ptr(verts), verts.shape[0],
                                       N.ptr(faces), faces.shape[0], N.ptr(record), N.stream_of(device)),
                "batch emit")

    def backward(self, normalize, exact, gv, record, vcap, fcap, device):
        N.check(_lib().diso_batch_backward(self.ex._h, int(bool(normalize)), N.GRAD_EXACT if exact else 0,
                                           N.ptr(gv), N.ptr(record), int(vcap), int(fcap), N.stream_of(device)),
                "batch backward")


def record_slots(grids):
    return int(_lib().diso_batch_record_slots(grids, len(grids)))


def _guard(res, i, iso, dtype):
    c = res.counts[i]
    isoS = N.iso_values(iso, dtype)[0]
    return c.sdf_min >= isoS or c.sdf_max <= isoS


class _BatchFunction(Function):
    @staticmethod
    def forward(ctx, bx, n, has_def, isos, normalize, return_quads, exact_grad, iso_grids, *inputs):
        # inputs: the n grids, the n deforms (has_def), then the isovalue tensors of
        # the grids listed in iso_grids (those whose isovalue requires grad)
        sdfs = [t.detach().contiguous() for t in inputs[:n]]
        defs = [t.detach().contiguous() for t in inputs[n:2 * n]] if has_def else None
        dev = sdfs[0].device
        grids = _grids(sdfs, defs, isos, bx.dtype)
        record = torch.empty(record_slots(grids), dtype=torch.int64, device=dev)
        bx.prepare(grids, record, dev)
        bx.count(dev)
        res = bx.results(n, dev)
        nv = int(res.voff[n - 1] + res.counts[n - 1].n_verts)
        nf = int(res.foff[n - 1] + res.counts[n - 1].n_faces)
        width = 3 if bx.method == N.MC else 4
        verts = torch.empty((nv, 3), dtype=bx.dtype, device=dev)
        faces = torch.empty((nf, width), dtype=torch.int64, device=dev)
        wants_grad = any(ctx.needs_input_grad[8:])
        edges = bx.edge_record(nv, nf, dev) if wants_grad else None
        bx.emit(normalize, verts, faces, dev, edges)
        ctx.bx, ctx.n, ctx.has_def, ctx.isos, ctx.normalize, ctx.exact = bx, n, has_def, isos, normalize, exact_grad
        ctx.record, ctx.edges, ctx.caps = record, edges, (nv, nf)
        ctx.iso_grids = iso_grids
        ctx.iso_like = [(t.dtype, t.device, t.shape) for t in inputs[(2 if has_def else 1) * n:]]
        ctx.save_for_backward(*inputs[:(2 if has_def else 1) * n])
        meta = [(int(res.voff[i]), int(res.counts[i].n_verts), int(res.foff[i]), int(res.counts[i].n_faces),
                 _guard(res, i, isos[i], bx.dtype)) for i in range(n)]
        ctx.meta = meta
        if bx.method == N.DMC and not return_quads:
            # the quad split orders each grid's faces on their own (config-1 pairs first)
            parts = []
            for (v0, nvi, f0, nfi, _), i in zip(meta, range(n)):
                q = faces[f0:f0 + nfi]
                t = torch.empty((2 * nfi, 3), dtype=torch.int64, device=dev)
                m = bx.ex.split(verts[v0:v0 + nvi], q, t) if nfi else 0
                parts.append(t[:m])
            faces = torch.cat(parts) if parts else faces.new_empty((0, 3))
            sizes = [p.shape[0] for p in parts]
            offs = [sum(sizes[:i]) for i in range(n)]
            ctx.meta = meta = [(v0, nvi, offs[i], sizes[i], g) for i, (v0, nvi, _, _, g) in enumerate(meta)]
        ctx.mark_non_differentiable(faces)
        bx.last_meta = meta  # per-grid (vertex offset, count, face offset, count, guard) for extract_batch
        return verts, faces

    @staticmethod
    def backward(ctx, gverts, gfaces):
        inputs = ctx.saved_tensors
        n = ctx.n
        sdfs = [t.detach().contiguous() for t in inputs[:n]]
        defs = [t.detach().contiguous() for t in inputs[n:2 * n]] if ctx.has_def else None
        dev = sdfs[0].device
        gs = [torch.empty_like(s) for s in sdfs]
        gd = [torch.empty_like(d) for d in defs] if defs is not None else None
        grids = _grids(sdfs, defs, ctx.isos, ctx.bx.dtype, gs, gd)
        bx = ctx.bx
        # the forward's records (scanned segment counts and tile bytes; the edge record)
        # are all the state kept
        bx.prepare(grids, ctx.record, dev)
        gv = gverts.contiguous() if gverts is not None else torch.zeros(0, 3, dtype=bx.dtype, device=dev)
        bx.backward(ctx.normalize, ctx.exact, gv, ctx.edges, *ctx.caps, dev)
        # dL/d(isovalue) per grid: minus the sum of the grid's dL/dsdf
        giso = [bx.ex.isovalue_grad(gs[i]).to(device=device, dtype=dtype).reshape(shape)
                for i, (dtype, device, shape) in zip(ctx.iso_grids, ctx.iso_like)]
        return (None,) * 8 + tuple(gs) + (tuple(gd) if gd is not None else ()) + tuple(giso)


def extract_batch(bx: _Batch, sdfs, deforms=None, isovalue=0.0, normalize=True, return_quads=False,
                  exact_grad=False):
    """Differentiable extraction of a list of grids; returns a list of (verts, faces),
    each what DiffMC / DiffDMC returns for that grid alone.  `isovalue`: one value
    for all grids or one per grid; a tensor that requires grad receives
    dL/d(isovalue)."""
    n = len(sdfs)
    if n == 0:
        return []
    isos = list(isovalue) if isinstance(isovalue, (list, tuple)) else [isovalue] * n
    if len(isos) != n:
        raise RuntimeError(f"{len(isos)} isovalues for {n} grids")
    iso_grids = [i for i, v in enumerate(isos)
                 if isinstance(v, torch.Tensor) and v.requires_grad and torch.is_grad_enabled()]
    for s in sdfs:
        if not s.is_cuda or s.dim() != 3 or s.dtype != bx.dtype:
            raise RuntimeError("every grid must be a 3-d CUDA tensor of the extractor's dtype")
    if deforms is not None:
        for s, d in zip(sdfs, deforms):
            if d is None or tuple(d.shape) != tuple(s.shape) + (3,) or d.dtype != bx.dtype:
                raise RuntimeError("deforms must be [X, Y, Z, 3] tensors matching their grids")
    inputs = list(sdfs) + (list(deforms) if deforms is not None else []) + [isos[i] for i in iso_grids]
    values = [float(v.detach()) if isinstance(v, torch.Tensor) else float(v) for v in isos]
    with torch.cuda.device(sdfs[0].device):
        verts, faces = _BatchFunction.apply(bx, n, deforms is not None, values, bool(normalize), bool(return_quads),
                                            bool(exact_grad), iso_grids, *inputs)
    out = []
    width = 3 if (bx.method == N.MC or not return_quads) else 4
    for i, (v0, nvi, f0, nfi, empty) in enumerate(bx.last_meta):
        if empty:
            out.append((torch.zeros((0, 3), dtype=bx.dtype, device=verts.device),
                        torch.zeros((0, 3 if bx.method == N.MC else 4), dtype=torch.int32, device=verts.device)))
        else:
            out.append((verts[v0:v0 + nvi], faces[f0:f0 + nfi].view(-1, width)))
    return out


class _BatchModule(nn.Module):
    METHOD = N.MC

    def __init__(self, dtype=torch.float32, *, exact_grad=False):
        super().__init__()
        self.dtype = dtype
        self.exact_grad = exact_grad
        self._bx = _Batch(self.METHOD, dtype)


class DiffMCBatch(_BatchModule):
    """Marching cubes over a list of grids (one launch per phase for all of them)."""

    METHOD = N.MC

    def forward(self, grids, deforms=None, isovalue=0.0, normalize=True):
        return extract_batch(self._bx, grids, deforms, isovalue, normalize, False)


class DiffDMCBatch(_BatchModule):
    """Dual marching cubes over a list of grids."""

    METHOD = N.DMC

    def forward(self, grids, deforms=None, isovalue=0.0, return_quads=False, normalize=True):
        return extract_batch(self._bx, grids, deforms, isovalue, normalize, return_quads, self.exact_grad)


class BatchPlan:
    """A fixed list of grid shapes with device-resident inputs, outputs and
    gradients, whose forward + backward is one CUDA graph.

    Fill ``plan.sdf[i]`` / ``plan.deform[i]`` in place and ``plan.grad_verts``
    (dL/dverts of the concatenated vertices, e.g. fixed loss weights), then
    ``replay()``; read sizes with ``results()`` (one synchronisation) and meshes
    with ``meshes()``.  Outputs have fixed capacities: ``results()`` raises when
    a replay overflowed them; ``size_outputs()`` re-sizes from a fresh count
    (and drops the captured graph).
    """

    def __init__(self, method, dtype, shapes, *, deform=True, isovalue=0.0, normalize=True, exact_grad=False,
                 device="cuda"):
        self.device = torch.device(device)
        self.method, self.dtype = method, dtype
        self.shapes = [tuple(s) for s in shapes]
        self.n = len(self.shapes)
        self.normalize, self.exact = bool(normalize), bool(exact_grad)
        self.isos = list(isovalue) if isinstance(isovalue, (list, tuple)) else [float(isovalue)] * self.n
        self.bx = _Batch(method, dtype)
        with torch.cuda.device(self.device):
            self.sdf = [torch.zeros(s, dtype=dtype, device=self.device) for s in self.shapes]
            self.deform = [torch.zeros(s + (3,), dtype=dtype, device=self.device) for s in self.shapes] if deform else None
            self.grad_sdf = [torch.empty(s, dtype=dtype, device=self.device) for s in self.shapes]
            self.grad_deform = ([torch.empty(s + (3,), dtype=dtype, device=self.device) for s in self.shapes]
                                if deform else None)
            grids = _grids(self.sdf, self.deform, self.isos, dtype, self.grad_sdf, self.grad_deform)
            self.record = torch.empty(record_slots(grids), dtype=torch.int64, device=self.device)
            self.bx.prepare(grids, self.record, self.device)
        self.verts = self.faces = self.grad_verts = None
        self.graph = None

    def size_outputs(self, margin=1.25, minimum=1024):
        """Count the current inputs and allocate outputs with `margin` headroom."""
        with torch.cuda.device(self.device):
            self.bx.count(self.device)
            r = self.bx.results(self.n, self.device)
            nv = int(r.voff[self.n - 1] + r.counts[self.n - 1].n_verts)
            nf = int(r.foff[self.n - 1] + r.counts[self.n - 1].n_faces)
            vcap, fcap = max(minimum, int(nv * margin)), max(minimum, int(nf * margin))
            width = 3 if self.method == N.MC else 4
            self.verts = torch.empty((vcap, 3), dtype=self.dtype, device=self.device)
            self.faces = torch.empty((fcap, width), dtype=torch.int64, device=self.device)
            self.grad_verts = torch.zeros((vcap, 3), dtype=self.dtype, device=self.device)
            self.edges = self.bx.edge_record(vcap, fcap, self.device)
        self.graph = None
        return nv, nf

    def run(self):
        """Count, emit and backward of every grid: device work only, no host synchronisation."""
        self.bx.count(self.device)
        self.bx.emit(self.normalize, self.verts, self.faces, self.device, self.edges)
        self.bx.backward(self.normalize, self.exact, self.grad_verts, self.edges, self.verts.shape[0],
                         self.faces.shape[0], self.device)

    def capture(self):
        if self.verts is None:
            self.size_outputs()
        with torch.cuda.device(self.device):
            s = torch.cuda.Stream()
            s.wait_stream(torch.cuda.current_stream())
            with torch.cuda.stream(s):
                self.run()  # warm-up outside the graph
            torch.cuda.current_stream().wait_stream(s)
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                self.run()
            torch.cuda.synchronize()
        self.graph = g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def results(self):
        with torch.cuda.device(self.device):
            r = self.bx.results(self.n, self.device)
        if r.overflow.value:
            raise RuntimeError("BatchPlan outputs overflowed their capacity; call size_outputs() and capture again")
        return r

    def meshes(self):
        """Per-grid (verts, faces) views of the last run, with the empty-surface guard applied."""
        r = self.results()
        out = []
        for i in range(self.n):
            c = r.counts[i]
            if _guard(r, i, self.isos[i], self.dtype):
                out.append((self.verts[:0], torch.zeros((0, self.faces.shape[1]), dtype=torch.int32,
                                                        device=self.device)))
            else:
                out.append((self.verts[r.voff[i]:r.voff[i] + c.n_verts], self.faces[r.foff[i]:r.foff[i] + c.n_faces]))
        return out
