"""Narrow-band input: a grid whose values are stored only in 8 x 8 x 8-point bricks
near the surface.

The reference takes dense [N, N, N] grids only (diso/__init__.py:48, 102), so its
grids stop where their dense arrays stop (32 B per point in fp32 with deform and both
gradients: 275 GB at 2048^3).  A ``BrickGrid`` keeps

* ``index`` [ceil(n0/8), ceil(n1/8), ceil(n2/8)] int32: each brick's slot, or
  BRICK_OUTSIDE (-1) / BRICK_INSIDE (-2) for an absent brick, whose points read
  +background / -background;
* ``values`` [K, 8, 8, 8] (z fastest) and optionally ``deform`` [K, 8, 8, 8, 3].

Its meshes are exactly those of the dense grid that ``dense()`` returns (absent bricks
filled with +-background, zero deform there): the same vertices, faces and order.
``extract_bricks`` runs the forward (diso_forward_bricks) and, through autograd, the
backward (diso_backward_bricks) into the slots: dL/dvalues and dL/ddeform are the
dense gradients at the bricks' points.  Memory grows with the bricks, the index (4 B
per brick) and the segment record (8 B per 32-cell row segment); DMC keeps its cell
records in the extractor's scratch only for the count units that hold the surface.
"""
from __future__ import annotations

import math

import torch
from torch.autograd import Function

from . import _native as N

B = N.BRICK


def brick_dims(dims):
    return tuple((int(n) + B - 1) // B for n in dims)


def _to_bricks(t, nb, fill):
    """[n0, n1, n2, *rest] -> [nb0 * nb1 * nb2, 8, 8, 8, *rest] in brick order (x-major),
    points beyond the grid set to `fill`."""
    rest = tuple(t.shape[3:])
    full = torch.full((nb[0] * B, nb[1] * B, nb[2] * B) + rest, fill, dtype=t.dtype, device=t.device)
    full[:t.shape[0], :t.shape[1], :t.shape[2]] = t
    perm = (0, 2, 4, 1, 3, 5) + tuple(range(6, 6 + len(rest)))
    return full.reshape(nb[0], B, nb[1], B, nb[2], B, *rest).permute(*perm).reshape(
        nb[0] * nb[1] * nb[2], B, B, B, *rest)


class BrickGrid:
    """A narrow band (see the module's docstring).  index, values and deform live on one
    device; values and deform share a dtype (float32 or float64)."""

    def __init__(self, dims, index, values, deform=None, background=1.0):
        self.dims = tuple(int(n) for n in dims)
        if len(self.dims) != 3 or min(self.dims) < 1:
            raise RuntimeError(f"dims must be three sizes >= 1, got {dims}")
        nb = brick_dims(self.dims)
        if index.dtype != torch.int32 or tuple(index.shape) != nb:
            raise RuntimeError(f"index must be int32 of shape {nb}, got {index.dtype} {tuple(index.shape)}")
        if values.dim() != 4 or tuple(values.shape[1:]) != (B, B, B) or values.dtype not in (torch.float32,
                                                                                             torch.float64):
            raise RuntimeError(f"values must be float32 / float64 [K, 8, 8, 8], got {values.dtype} "
                               f"{tuple(values.shape)}")
        if values.device != index.device:
            raise RuntimeError("index and values must be on one device")
        if deform is not None and (tuple(deform.shape) != tuple(values.shape) + (3,) or deform.dtype != values.dtype
                                   or deform.device != values.device):
            raise RuntimeError("deform must be [K, 8, 8, 8, 3] of the values' dtype and device")
        background = float(background)
        if not math.isfinite(background) or background <= 0:
            raise RuntimeError(f"background must be finite and > 0, got {background}")
        self.index = index.contiguous()
        self.values = values
        self.deform = deform
        self.background = background

    @property
    def device(self):
        return self.values.device

    @property
    def dtype(self):
        return self.values.dtype

    @property
    def count(self):
        return int(self.values.shape[0])

    @classmethod
    def from_dense(cls, sdf, isovalue=0.0, band=0.0, deform=None, background=None):
        """The band of a dense grid: every brick that holds an end point of a crossing
        edge (the edges to the virtual pad, whose value is >= isovalue, included) or a
        point within `band` of isovalue; the other bricks are absent, tagged by their
        side.  With background > |isovalue| (the default: 2 |isovalue| + 1, or more)
        every point keeps its side of isovalue, so the band's meshes are the dense
        grid's, vertex for vertex."""
        if sdf.dim() != 3:
            raise RuntimeError("sdf must be [n0, n1, n2]")
        iso = float(isovalue)
        bg = float(background) if background is not None else 2.0 * abs(iso) + 1.0
        n = tuple(sdf.shape)
        nb = brick_dims(n)
        side = sdf >= iso
        mark = (sdf - iso).abs() <= float(band)
        for a in range(3):
            if n[a] > 1:
                d = side.narrow(a, 1, n[a] - 1) != side.narrow(a, 0, n[a] - 1)
                mark.narrow(a, 1, n[a] - 1).logical_or_(d)
                mark.narrow(a, 0, n[a] - 1).logical_or_(d)
            # the edges to the pad (iso + 1) from the faces' points below iso
            mark.narrow(a, 0, 1).logical_or_(~side.narrow(a, 0, 1))
            mark.narrow(a, n[a] - 1, 1).logical_or_(~side.narrow(a, n[a] - 1, 1))
        present = _to_bricks(mark, nb, False).flatten(1).any(1)
        above = _to_bricks(side, nb, False).flatten(1).any(1)
        slots = torch.cumsum(present.to(torch.int64), 0) - 1
        index = torch.where(present, slots, torch.where(above, N.BRICK_OUTSIDE, N.BRICK_INSIDE))
        index = index.to(torch.int32).reshape(nb)
        values = _to_bricks(sdf, nb, bg)[present].contiguous()
        dfm = _to_bricks(deform, nb, 0.0)[present].contiguous() if deform is not None else None
        return cls(n, index, values, dfm, bg)

    def dense(self):
        """The dense grid [n0, n1, n2] (and deform [n0, n1, n2, 3] or None) whose meshes
        the band's are: absent bricks read +-background, zero deform."""
        nb = brick_dims(self.dims)
        idx = self.index.reshape(-1).to(torch.int64)
        hi = torch.tensor(self.background, dtype=self.dtype, device=self.device)
        full = torch.where(idx == N.BRICK_INSIDE, -hi, hi)
        grid = full[:, None, None, None].expand(idx.shape[0], B, B, B).clone()
        pres = idx >= 0
        grid[pres] = self.values.detach()[idx[pres]]
        grid = grid.reshape(nb[0], nb[1], nb[2], B, B, B).permute(0, 3, 1, 4, 2, 5).reshape(
            nb[0] * B, nb[1] * B, nb[2] * B)[:self.dims[0], :self.dims[1], :self.dims[2]].contiguous()
        if self.deform is None:
            return grid, None
        d = torch.zeros((idx.shape[0], B, B, B, 3), dtype=self.dtype, device=self.device)
        d[pres] = self.deform.detach()[idx[pres]]
        d = d.reshape(nb[0], nb[1], nb[2], B, B, B, 3).permute(0, 3, 1, 4, 2, 5, 6).reshape(
            nb[0] * B, nb[1] * B, nb[2] * B, 3)[:self.dims[0], :self.dims[1], :self.dims[2]].contiguous()
        return grid, d

    def desc(self, values=None, deform=None):
        """The C descriptor (the tensors it points to are kept alive on self)."""
        v = (self.values if values is None else values).contiguous()
        d = self.deform if deform is None else deform
        d = d.contiguous() if d is not None else None
        self._keep = (v, d)
        c = N.BrickGridDesc()
        c.dims[:] = self.dims
        c.index = self.index.data_ptr()
        c.count = v.shape[0]
        c.values = v.data_ptr() if v.numel() else None
        c.deform = d.data_ptr() if d is not None and d.numel() else None
        c.background = self.background
        return c

    def materialize(self):
        """dense() computed by the library's kernel (CUDA tensors only)."""
        if not self.device.type == "cuda":
            raise RuntimeError("materialize needs CUDA tensors (dense() works anywhere)")
        sdf = torch.empty(self.dims, dtype=self.dtype, device=self.device)
        dfm = torch.empty(self.dims + (3,), dtype=self.dtype, device=self.device) if self.deform is not None else None
        with torch.cuda.device(self.device):
            N.check(N.lib().diso_bricks_materialize(N.dtype_tag(self.dtype), N.ctypes.byref(self.desc()), N.ptr(sdf),
                                                    N.ptr(dfm), N.stream_of(self.device)), "bricks materialize")
        return sdf, dfm


def _capacity(n):
    return n + n // 8 + 1024


class _BrickFunction(Function):
    """Autograd node of one narrow-band extraction: the forward has run (its `seg`
    record is kept); the backward gives dL/dvalues and dL/ddeform in the slots."""

    @staticmethod
    def forward(ctx, values, deform, ex, grid, iso, pad, normalize, exact, seg, verts, faces):
        ctx.ex, ctx.grid, ctx.iso, ctx.pad, ctx.normalize, ctx.exact = ex, grid, iso, pad, normalize, exact
        ctx.has_deform = deform is not None
        ctx.save_for_backward(seg, values, deform if deform is not None else seg.new_empty(0))
        ctx.mark_non_differentiable(faces)
        ctx.set_materialize_grads(False)
        ctx.nv = verts.shape[0]
        return verts, faces

    @staticmethod
    def backward(ctx, grad_verts, grad_faces):
        seg, values, deform = ctx.saved_tensors
        ex, grid = ctx.ex, ctx.grid
        dev = seg.device
        with torch.cuda.device(dev):
            if grad_verts is None:
                grad_verts = torch.zeros((ctx.nv, 3), dtype=ex.dtype, device=dev)
            v = values.detach().contiguous()
            d = deform.detach().contiguous() if ctx.has_deform else None
            gval = torch.empty_like(v)
            gd = torch.empty_like(d) if d is not None else None
            ex.backward_bricks(grid.desc(v, d), ctx.iso, ctx.pad, seg, ctx.normalize, grad_verts.contiguous(), gval,
                               gd, ctx.exact)
        return (gval if ctx.needs_input_grad[0] else None, gd if ctx.needs_input_grad[1] else None,
                None, None, None, None, None, None, None, None, None)


def extract_bricks(ex: N.Extractor, grid: BrickGrid, isovalue=0.0, normalize=True, return_quads=False,
                   exact_grad=False):
    """The mesh of a narrow band with the reference's semantics for the dense grid
    grid.dense() (empty-surface guard included); differentiable with respect to
    grid.values and grid.deform when they require grad (exact_grad as for DiffDMC)."""
    if grid.dtype != ex.dtype:
        raise RuntimeError(f"the band's dtype {grid.dtype} is not the extractor's {ex.dtype}")
    if grid.device.type != "cuda":
        raise RuntimeError("the band must be on a CUDA device")
    iso, pad = N.iso_values(isovalue, ex.dtype)
    width = 3 if ex.method == N.MC else 4
    dev = grid.device
    dims = grid.dims
    wants_grad = torch.is_grad_enabled() and (grid.values.requires_grad or
                                              (grid.deform is not None and grid.deform.requires_grad))
    with torch.cuda.device(dev):
        v = grid.values.detach().contiguous()
        d = grid.deform.detach().contiguous() if grid.deform is not None else None
        desc = grid.desc(v, d)
        seg = torch.empty(N.Extractor.segment_slots(dims), dtype=torch.int64, device=dev)
        hints = ex.brick_hints
        key = (dims, grid.count)
        vcap, fcap = hints.get(key, (1 << 16, 1 << 16))
        while True:
            verts = torch.empty((vcap, 3), dtype=ex.dtype, device=dev)
            faces = torch.empty((fcap, width), dtype=torch.int64, device=dev)
            counts = ex.forward_bricks(desc, iso, pad, seg, normalize, verts, faces)
            nv, nf = int(counts.n_verts), int(counts.n_faces)
            hints[key] = (_capacity(nv), _capacity(nf))
            if counts.empty:
                return (torch.zeros((0, 3), dtype=ex.dtype, device=dev),
                        torch.zeros((0, width), dtype=torch.int32, device=dev))
            if counts.emitted:
                break
            vcap, fcap = nv, nf
        verts, faces = verts[:nv], faces[:nf]
        if ex.method == N.DMC and not return_quads:
            tris = torch.empty((2 * nf, 3), dtype=torch.int64, device=dev)
            faces = tris[:ex.split(verts, faces, tris)]
        if not wants_grad:
            return verts, faces
        return _BrickFunction.apply(grid.values, grid.deform, ex, grid, iso, pad, bool(normalize), bool(exact_grad),
                                    seg, verts, faces)
