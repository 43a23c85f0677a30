"""Fields evaluated by the extractor instead of a dense grid.

The reference's caller evaluates its SDF on a full meshgrid in PyTorch and hands the
dense [N, N, N] tensor to DiffMC / DiffDMC (test/example.py:8-16, 33-53).  A field
given to ``DiffMC.forward_field`` / ``DiffDMC.forward_field`` is evaluated where the
extractor needs values: the count evaluates only the chunks of 8 x 32 x 32 cells that
may hold the surface (the others it classifies whole from bounds of the field), the
emit evaluates the end points of the crossing edges.  The mesh equals that of the
dense path on ``field.materialize(shape)``, bit for bit.

With a deform (a dense [N, N, N, 3] tensor, as for a dense grid) and centres, radii or
deform that require grad, the mesh is differentiable: the backward
(diso_backward_field) recomputes the crossings near the surface from the field, and
each grid point's dL/d(value) goes to the sphere attaining the minimum there, so the
gradients of the centres and radii come without a dense grid of the field's values.
"""
from __future__ import annotations

import torch
from torch.autograd import Function

from . import _native as N


class SphereUnion:
    """value(p) = min_k (|p - c_k| - r_k) at the grid points
    p = lo + (hi - lo) * i / (n - 1) per axis; the reference example's SphereSDF is
    the one-sphere case.  centers [K, 3] and radii [K] are CUDA tensors."""

    def __init__(self, centers, radii, lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0)):
        c = torch.as_tensor(centers)
        r = torch.as_tensor(radii)
        if not c.is_cuda or r.device != c.device:
            raise RuntimeError("centers and radii must be CUDA tensors on one device")
        if c.dim() != 2 or c.shape[1] != 3 or r.dim() != 1 or r.shape[0] != c.shape[0] or c.shape[0] < 1:
            raise RuntimeError("centers must be [K, 3] and radii [K] with K >= 1")
        self.centers, self.radii = c, r  # differentiable through extract_field when they require grad
        self.spheres = torch.cat([c.detach(), r.detach().to(c.dtype)[:, None]], 1).contiguous()
        self.lo = tuple(float(x) for x in lo)
        self.hi = tuple(float(x) for x in hi)
        if len(self.lo) != 3 or len(self.hi) != 3:
            raise RuntimeError("lo and hi need three coordinates")

    @property
    def device(self):
        return self.spheres.device

    def desc(self, dtype, deform=None):
        """The C descriptor, with the spheres in `dtype` (kept alive on self) and the
        deform [n0, n1, n2, 3] or None."""
        sph = self.spheres if self.spheres.dtype == dtype else self.spheres.to(dtype).contiguous()
        self._desc_spheres = sph
        d = N.SphereFieldDesc()
        d.spheres = sph.data_ptr()
        d.count = sph.shape[0]
        d.lo[:] = self.lo
        d.hi[:] = self.hi
        d.deform = None if deform is None else deform.data_ptr()
        return d

    @property
    def requires_grad(self):
        return self.centers.requires_grad or self.radii.requires_grad

    def materialize(self, shape, dtype=torch.float32):
        """The dense grid [n0, n1, n2] of the field (the values the fused path evaluates)."""
        shape = tuple(int(n) for n in shape)
        out = torch.empty(shape, dtype=dtype, device=self.device)
        with torch.cuda.device(self.device):
            N.check(N.lib().diso_field_materialize(N.dtype_tag(dtype), N.ctypes.byref(self.desc(dtype)), *shape,
                                                   N.ptr(out), N.stream_of(self.device)), "field materialize")
        return out


def _capacity(n):
    return n + n // 8 + 1024


class _FieldFunction(Function):
    """Autograd node of one extraction of an evaluated field: the forward has run (its
    `seg` record is kept); the backward gives dL/d(centres, radii) and dL/ddeform."""

    @staticmethod
    def forward(ctx, centers, radii, deform, ex, field, shape, iso, pad, normalize, exact, seg, verts, faces):
        ctx.ex, ctx.field, ctx.shape, ctx.iso, ctx.pad = ex, field, shape, iso, pad
        ctx.normalize, ctx.exact = normalize, exact
        ctx.has_deform = deform is not None
        ctx.save_for_backward(seg, deform if deform is not None else seg.new_empty(0))
        ctx.mark_non_differentiable(faces)
        ctx.set_materialize_grads(False)
        ctx.nv = verts.shape[0]
        return verts, faces

    @staticmethod
    def backward(ctx, grad_verts, grad_faces):
        seg, deform = ctx.saved_tensors
        ex, field = ctx.ex, ctx.field
        dev = seg.device
        with torch.cuda.device(dev):
            if grad_verts is None:
                grad_verts = torch.zeros((ctx.nv, 3), dtype=ex.dtype, device=dev)
            gv = grad_verts.contiguous()
            d = deform.detach().contiguous() if ctx.has_deform else None
            gd = torch.empty_like(d) if d is not None else None
            gsph = torch.empty((field.spheres.shape[0], 4), dtype=torch.float64, device=dev)
            ex.backward_field(field.desc(ex.dtype, d), ctx.shape, ctx.iso, ctx.pad, seg, ctx.normalize, gv, gsph, gd,
                              ctx.exact)
        gc = gsph[:, :3].to(field.centers.dtype) if ctx.needs_input_grad[0] else None
        gr = gsph[:, 3].to(field.radii.dtype) if ctx.needs_input_grad[1] else None
        return gc, gr, gd, None, None, None, None, None, None, None, None, None, None


def extract_field(ex: N.Extractor, field, shape, isovalue=0.0, normalize=True, return_quads=False, deform=None,
                  exact_grad=False):
    """The mesh of `field` on a grid of `shape`, with the reference's semantics for the
    same values on a dense grid (empty-surface guard included).  `deform` [n0, n1,
    n2, 3] moves the vertices as for a dense grid.  When the field's centres or radii
    (or the deform) require grad, the vertices are differentiable with respect to
    them (exact_grad as for DiffDMC)."""
    shape = tuple(int(n) for n in shape)
    if len(shape) != 3 or min(shape) < 1:
        raise RuntimeError(f"shape must be three sizes >= 1, got {shape}")
    if deform is not None:
        if tuple(deform.shape) != shape + (3,) or deform.dtype != ex.dtype or deform.device != field.device:
            raise RuntimeError(f"deform must be {shape + (3,)} of the extractor's dtype on the field's device")
    iso, pad = N.iso_values(isovalue, ex.dtype)
    width = 3 if ex.method == N.MC else 4
    dev = field.device
    wants_grad = torch.is_grad_enabled() and (field.requires_grad or (deform is not None and deform.requires_grad))
    d = deform.detach().contiguous() if deform is not None else None
    with torch.cuda.device(dev):
        desc = field.desc(ex.dtype, d)
        seg = torch.empty(N.Extractor.segment_slots(shape), dtype=torch.int64, device=dev)
        hints = ex.field_hints
        vcap, fcap = hints.get(shape, (1 << 16, 1 << 16))
        while True:
            verts = torch.empty((vcap, 3), dtype=ex.dtype, device=dev)
            faces = torch.empty((fcap, width), dtype=torch.int64, device=dev)
            counts = ex.forward_field(desc, shape, iso, pad, seg, normalize, verts, faces)
            nv, nf = int(counts.n_verts), int(counts.n_faces)
            hints[shape] = (_capacity(nv), _capacity(nf))
            if counts.empty:
                return (torch.zeros((0, 3), dtype=ex.dtype, device=dev),
                        torch.zeros((0, width), dtype=torch.int32, device=dev))
            if counts.emitted:
                break
            vcap, fcap = _capacity(nv), _capacity(nf)
        verts, faces = verts[:nv], faces[:nf]
        if ex.method == N.DMC and not return_quads:
            tris = torch.empty((2 * nf, 3), dtype=torch.int64, device=dev)
            faces = tris[:ex.split(verts, faces, tris)]
        if not wants_grad:
            return verts, faces
        return _FieldFunction.apply(field.centers, field.radii, deform, ex, field, shape, iso, pad, bool(normalize),
                                    bool(exact_grad), seg, verts, faces)
