"""DiffMC / DiffDMC: drop-in replacements of the reference's nn.Modules
(diso/__init__.py:9-147) over the native extractor.

Differences that are invisible to callers of the reference API:

* the one-voxel pad (diso/__init__.py:52-54) is virtual, so no padded copies of
  the grid or the deform are made, and the gradients come back unpadded
  directly;
* the empty-surface guard (diso/__init__.py:49, 103) reuses the min/max that the
  counting kernel computes, so a forward synchronises with the host once (the
  reference syncs for min, max and three output sizes);
* the backward does not re-run the forward (diso/__init__.py:32, 86): the
  forward records every crossing edge (its cell and axis, for DMC the patches
  around it) when a gradient will be wanted and zeroes the gradient buffers beside
  its count; the backward computes each edge's adjoint once and writes the
  gradients near the surface, deterministically (no atomics);
* vertices are shifted and normalised, and faces written as int64, inside the
  kernels; the DMC quad split runs on the GPU in one pass plus a scan;
* an isovalue given as a tensor that requires grad gets dL/d(isovalue), minus
  the sum of dL/dsdf (the reference's isovalue is a plain scalar).

By default (recompute=True, as the reference, which re-runs its forward in its
backward, diso/__init__.py:32, 86) the forward keeps nothing for the backward but
the inputs and its segment record (the scanned output counts per 32-cell row
segment, 8 bytes per 32 cells): no edge record and no gradient buffers.  The
backward recomputes the crossings, the DMC cell codes and patch ids and every
edge's adjoint per point tile in one pass that writes each gradient element once
(diso_backward_recompute).  recompute=False keeps the edge record and the zeroed
gradient buffers from the forward instead (a faster backward for 2.4 GB more
device memory between the two at 512^3 with deform); the gradients are the same
bit for bit.

The outputs are the reference's: the same vertex, face and quad order, the same
dtypes, including the int32 empty faces of the guard.
"""
from __future__ import annotations

import torch
from torch import nn
from torch.autograd import Function

from . import _native as N

# Optional phase timer: when set to a callable, it is called as timer(name, "start"
# | "end") around each native phase (forward, split, backward) on the current
# stream; bench.py uses it to record CUDA events inside its timed region.
phase_timer = None


def _mark(name, what):
    if phase_timer is not None:
        phase_timer(name, what)


def _check_inputs(grid, deform, dtype):
    if not grid.is_cuda:
        raise RuntimeError("grid must be a CUDA tensor")
    if grid.dim() != 3:
        raise RuntimeError(f"grid must be [X, Y, Z], got shape {tuple(grid.shape)}")
    if grid.dtype != dtype:
        raise RuntimeError("grid type must match the mc class")
    if deform is not None:
        if not deform.is_cuda or deform.device != grid.device:
            raise RuntimeError("deform must be a CUDA tensor on the grid's device")
        if deform.dtype != dtype:
            raise RuntimeError("deformation type must match the mc class")
        if tuple(deform.shape) != tuple(grid.shape) + (3,):
            raise RuntimeError(f"deform must be [X, Y, Z, 3], got {tuple(deform.shape)}")


class _ExtractFunction(Function):
    """Autograd node of one extraction; the counterpart of DMCFunction /
    DDMCFunction (diso/__init__.py:18-46, 72-100).  The forward's kernels have run
    when it is applied (extract below); it returns the outputs and keeps what the
    backward needs."""

    @staticmethod
    def forward(ctx, grid, deform, ex, seg, counts, iso, pad, normalize, return_quads, exact_grad, grads, out,
                iso_tensor, recompute):
        verts_buf, faces_buf, record = out
        nv, nf = int(counts.n_verts), int(counts.n_faces)
        verts, faces = verts_buf[:nv], faces_buf[:nf]
        if ex.method == N.DMC and not return_quads:
            tris = torch.empty((2 * nf, 3), dtype=torch.int64, device=verts.device)
            _mark("split", "start")
            n = ex.split(verts, faces, tris)
            _mark("split", "end")
            faces = tris[:n]
        wants_grad = ctx.needs_input_grad[0] or ctx.needs_input_grad[1] or ctx.needs_input_grad[12]
        ctx.iso_like = (iso_tensor.dtype, iso_tensor.device, iso_tensor.shape) if iso_tensor is not None else None
        ctx.gs, ctx.gd = grads if (wants_grad and grads is not None) else (None, None)
        ctx.ex = ex
        ctx.iso, ctx.pad, ctx.normalize, ctx.exact_grad = iso, pad, normalize, exact_grad
        ctx.has_deform = deform is not None
        ctx.recompute, ctx.counts = recompute, (nv, nf)
        ctx.save_for_backward(grid, deform if deform is not None else grid.new_empty(0), seg,
                              record if record is not None else seg.new_empty(0))
        ctx.mark_non_differentiable(faces)
        # the faces never get a gradient; without this autograd would fill one with zeros
        ctx.set_materialize_grads(False)
        return verts, faces

    @staticmethod
    def backward(ctx, grad_verts, grad_faces):
        grid, deform, seg, record = ctx.saved_tensors
        g = grid.detach().contiguous()
        d = deform.detach().contiguous() if ctx.has_deform else None
        with torch.cuda.device(g.device):
            if grad_verts is None:
                grad_verts = torch.zeros(ctx.counts[0], 3, dtype=g.dtype, device=g.device)
            gv = grad_verts.contiguous()
            _mark("backward", "start")
            if ctx.recompute:
                gs = torch.empty_like(g)
                gd = torch.empty_like(d) if d is not None else None
                ctx.ex.backward_recompute(g, d, ctx.iso, ctx.pad, seg, ctx.normalize, gv, gs, gd, ctx.exact_grad)
            else:
                gs, gd = ctx.gs, ctx.gd
                zeroed = gs is not None
                if not zeroed:  # a second backward of the same graph (retain_graph)
                    gs = torch.empty_like(g)
                    gd = torch.empty_like(d) if d is not None else None
                ctx.gs = ctx.gd = None
                ctx.ex.backward(g, d, ctx.iso, ctx.pad, seg, record, ctx.normalize, gv, gs, gd, ctx.exact_grad,
                                zeroed=zeroed)
            giso = None
            if ctx.needs_input_grad[12]:
                dtype, device, shape = ctx.iso_like
                giso = ctx.ex.isovalue_grad(gs, seg).to(device=device, dtype=dtype).reshape(shape)
            _mark("backward", "end")
        return gs, gd, None, None, None, None, None, None, None, None, None, None, giso, None


def _capacity(n):
    return n + n // 8 + 1024


def extract(ex: N.Extractor, grid, deform=None, isovalue=0.0, normalize=True, return_quads=False,
            exact_grad=False, recompute=True):
    """One differentiable extraction with the reference's semantics.

    An isovalue given as a tensor that requires grad (a one-element tensor, not in
    the reference) receives dL/d(isovalue) in the backward.

    recompute=True (the default) keeps no edge record and no gradient buffers
    between the forward and the backward, only the segment record; the backward
    recomputes the crossing lists per point tile.  recompute=False keeps them.

    exact_grad (DMC only) replaces the reference's backward in cells with several
    patches, where every patch receives the first patch's gradient
    (src/cudualmc.cu:990), by the true derivative.

    When the extractor has seen a grid of this shape before, the forward is one
    native call (count, scan and emit with no host round trip in between) into
    outputs sized from the last result with some headroom; the returned tensors
    are views of them.  Otherwise, or when they do not fit, the emit follows the
    count into outputs of the exact sizes."""
    _check_inputs(grid, deform, ex.dtype)
    iso, pad = N.iso_values(isovalue, ex.dtype)
    width = 3 if ex.method == N.MC else 4
    with torch.cuda.device(grid.device):
        dev = grid.device
        g = grid.detach().contiguous()
        d = deform.detach().contiguous() if deform is not None else None
        seg = torch.empty(N.Extractor.segment_slots(g.shape), dtype=torch.int64, device=dev)
        iso_tensor = isovalue if isinstance(isovalue, torch.Tensor) and isovalue.requires_grad else None
        wants_grad = torch.is_grad_enabled() and (grid.requires_grad or (deform is not None and deform.requires_grad)
                                                  or iso_tensor is not None)
        # When a gradient can be asked for, its buffers are allocated now; the forward's
        # count and emit write their zeros between their own loads (they leave HBM
        # bandwidth unused), and the backward writes only the point tiles near the
        # surface.
        keep = wants_grad and not recompute  # the edge record and the gradient buffers
        grads = None
        if keep:
            grads = (torch.empty_like(g), torch.empty(tuple(g.shape) + (3,), dtype=g.dtype, device=dev)
                     if d is not None else None)
            ex.zero_grads(*grads)
        hints = ex.size_hints
        hint = hints.get(tuple(g.shape))
        counts, out = None, None
        _mark("forward", "start")
        if hint is not None:
            vcap, fcap = hint
            verts = torch.empty((vcap, 3), dtype=ex.dtype, device=dev)
            faces = torch.empty((fcap, width), dtype=torch.int64, device=dev)
            record = (torch.empty(max(1, ex.record_slots(n_verts=vcap, n_faces=fcap)), dtype=torch.int64, device=dev)
                      if keep else None)
            counts = ex.forward(g, d, iso, pad, seg, normalize, verts, faces, record)
            if counts.emitted:
                out = (verts, faces, record)
        else:
            counts = ex.count(g, iso, pad, seg)
        hints[tuple(g.shape)] = (_capacity(int(counts.n_verts)), _capacity(int(counts.n_faces)))
        if counts.empty:
            _mark("forward", "end")
            return (torch.zeros((0, 3), dtype=ex.dtype, device=dev),
                    torch.zeros((0, width), dtype=torch.int32, device=dev))
        if out is None:
            nv, nf = int(counts.n_verts), int(counts.n_faces)
            verts = torch.empty((nv, 3), dtype=ex.dtype, device=dev)
            faces = torch.empty((nf, width), dtype=torch.int64, device=dev)
            record = (torch.empty(max(1, ex.record_slots(counts)), dtype=torch.int64, device=dev)
                      if keep else None)
            ex.emit(g, d, iso, pad, seg, normalize, verts, faces, record)
            out = (verts, faces, record)
        _mark("forward", "end")
        return _ExtractFunction.apply(grid, deform, ex, seg, counts, iso, pad, bool(normalize), bool(return_quads),
                                      bool(exact_grad), grads, out, iso_tensor, bool(recompute))


class DiffMC(nn.Module):
    """Differentiable marching cubes (diso/__init__.py:9-61).

    ``recompute`` (keyword only, not in the reference): True (the default) keeps
    nothing between the forward and the backward but the inputs and the segment
    record, and the backward recomputes the crossing lists; False keeps the edge
    record and the gradient buffers (a faster backward, more memory held)."""

    def __init__(self, dtype=torch.float32, *, recompute=True):
        super().__init__()
        self.dtype = dtype
        self.recompute = recompute
        self._ex = N.Extractor(N.MC, dtype)

    def forward(self, grid, deform=None, isovalue=0.0, normalize=True):
        return extract(self._ex, grid, deform, isovalue, normalize, recompute=self.recompute)

    def forward_field(self, field, shape, isovalue=0.0, normalize=True, deform=None):
        """The mesh of an evaluated field (diso_gb300.fields) on a grid of `shape`,
        without a dense grid in memory; differentiable with respect to the field's
        parameters and the deform."""
        from .fields import extract_field

        return extract_field(self._ex, field, shape, isovalue, normalize, deform=deform)

    def forward_bricks(self, grid, isovalue=0.0, normalize=True):
        """The mesh of a narrow band (diso_gb300.bricks.BrickGrid): that of its dense
        grid, without the dense grid in memory; differentiable with respect to
        grid.values and grid.deform."""
        from .bricks import extract_bricks

        return extract_bricks(self._ex, grid, isovalue, normalize)

    def forward_mlp(self, field, shape, isovalue=0.0, normalize=True):
        """The mesh of an MLP field (diso_gb300.neural.MLPField) on a grid of `shape`,
        from the narrow band where the network can cross the isovalue; differentiable
        with respect to the network's parameters."""
        from .neural import extract_mlp

        return extract_mlp(self._ex, field, shape, isovalue, normalize)


class DiffDMC(nn.Module):
    """Differentiable dual marching cubes (diso/__init__.py:63-147).

    ``exact_grad=True`` (keyword only, not in the reference) gives the true
    derivative in cells with several patches; the default reproduces the
    reference's gradient there (every patch gets the first patch's gradient).
    ``recompute=True`` as for DiffMC."""

    def __init__(self, dtype=torch.float32, *, exact_grad=False, recompute=True):
        super().__init__()
        self.dtype = dtype
        self.exact_grad = exact_grad
        self.recompute = recompute
        self._ex = N.Extractor(N.DMC, dtype)

    def forward(self, grid, deform=None, isovalue=0.0, return_quads=False, normalize=True):
        return extract(self._ex, grid, deform, isovalue, normalize, return_quads, self.exact_grad, self.recompute)

    def forward_field(self, field, shape, isovalue=0.0, return_quads=False, normalize=True, deform=None):
        """The mesh of an evaluated field (diso_gb300.fields) on a grid of `shape`,
        without a dense grid in memory; differentiable with respect to the field's
        parameters and the deform."""
        from .fields import extract_field

        return extract_field(self._ex, field, shape, isovalue, normalize, return_quads, deform, self.exact_grad)

    def forward_bricks(self, grid, isovalue=0.0, return_quads=False, normalize=True):
        """The mesh of a narrow band (diso_gb300.bricks.BrickGrid), as DiffMC.forward_bricks."""
        from .bricks import extract_bricks

        return extract_bricks(self._ex, grid, isovalue, normalize, return_quads, self.exact_grad)

    def forward_mlp(self, field, shape, isovalue=0.0, return_quads=False, normalize=True):
        """The mesh of an MLP field (diso_gb300.neural.MLPField), as DiffMC.forward_mlp."""
        from .neural import extract_mlp

        return extract_mlp(self._ex, field, shape, isovalue, normalize, return_quads, self.exact_grad)
