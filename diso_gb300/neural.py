"""MLP fields: a neural SDF evaluated only where the surface can be, then extracted
from the narrow band it fills.

The reference's caller evaluates its SDF on a full meshgrid and hands the dense
[N, N, N] tensor to DiffMC / DiffDMC (test/example.py:8-16, 33-53); for a neural SDF
that is N^3 network evaluations and an N^3 tensor.  ``MLPField`` evaluates the network
at the centres of the grid's 8^3-point bricks first, keeps the bricks that the
network's Lipschitz bound cannot rule out, evaluates the network at those bricks'
points only (matrix products on the tensor cores) and hands the band to the extractor
(``diso_gb300.bricks``).  Gradients reach the network's parameters through autograd:
the extractor's backward gives dL/d(value) at the bricks' points, and each chunk of
points is evaluated again in the backward (checkpointing), so the activations of all
the band's points are never held at once.

The band is exact, not a heuristic: an absent brick is one where the network provably
stays on one side of the isovalue over the brick and one grid step around it, so
every crossing edge has both end points in present bricks and the mesh equals that of
the dense grid of the network's values (up to the rounding of evaluating a point
inside one batch or another).  The proof is interval bound propagation through the
layers (Linear layers and monotone activations: each box's centre and radius pushed
through W and |W|, the activations applied to the interval's ends), in float64, one
box per brick; other networks need a Lipschitz bound (``lipschitz=``), and a brick is
then absent when its centre value lies farther from the isovalue than the bound times
the box's half diagonal.
"""
from __future__ import annotations

import math

import torch
from torch import nn
from torch.utils.checkpoint import checkpoint

from . import _native as N
from .bricks import BrickGrid, brick_dims

B = N.BRICK
ACTIVATIONS = (nn.ReLU, nn.Softplus, nn.LeakyReLU, nn.Tanh, nn.Sigmoid)  # monotone non-decreasing


class MLPField:
    """f(p) = net(p) at the grid points p = lo + (hi - lo) * i / (n - 1) per axis.

    ``net`` maps [M, 3] points to [M] or [M, 1] values.  An nn.Sequential of nn.Linear
    layers and monotone activations (ReLU, LeakyReLU with a slope >= 0, Softplus, Tanh,
    Sigmoid) is bounded over each brick by interval propagation; any other network
    needs ``lipschitz``, a bound on its Lipschitz constant over the domain."""

    def __init__(self, net, lo=(-1.0, -1.0, -1.0), hi=(1.0, 1.0, 1.0), lipschitz=None, chunk=1 << 20):
        self.net = net
        self.lo = tuple(float(x) for x in lo)
        self.hi = tuple(float(x) for x in hi)
        self._lip = lipschitz
        self.chunk = int(chunk)

    def propagable(self) -> bool:
        return isinstance(self.net, nn.Sequential) and all(
            isinstance(m, (nn.Linear,) + ACTIVATIONS) and not (isinstance(m, nn.LeakyReLU) and m.negative_slope < 0)
            for m in self.net)

    def bounds(self, lo, hi):
        """Lower and upper bounds [M] (float64) of the network over the boxes
        [lo, hi] ([M, 3] world coordinates), by interval propagation."""
        mu, r = (lo + hi) * 0.5, (hi - lo) * 0.5
        for m in self.net:
            if isinstance(m, nn.Linear):
                w = m.weight.detach().double()
                mu = mu @ w.t() + (m.bias.detach().double() if m.bias is not None else 0.0)
                r = r @ w.abs().t()
            else:  # monotone: the interval's ends map to the image's ends
                a, b = m(mu - r), m(mu + r)
                mu, r = (a + b) * 0.5, (b - a) * 0.5
        return (mu - r).reshape(-1), (mu + r).reshape(-1)

    def _steps(self, shape):
        return [((h - l) / (n - 1) if n > 1 else 0.0) for l, h, n in zip(self.lo, self.hi, shape)]

    def _eval(self, p):
        """The network at world points p [M, 3] (float64), in the network's dtype."""
        w = next(self.net.parameters())
        return self.net(p.to(w.dtype)).reshape(p.shape[0])

    def points(self, idx, shape):
        """World coordinates [M, 3] (float64) of grid points idx [M, 3] (integer or not)."""
        st = torch.tensor(self._steps(shape), dtype=torch.float64, device=idx.device)
        lo = torch.tensor(self.lo, dtype=torch.float64, device=idx.device)
        return lo + idx.to(torch.float64) * st

    def dense(self, shape, dtype=torch.float32, device=None):
        """The network's values on the whole grid (for checking; N^3 evaluations)."""
        device = device or next(self.net.parameters()).device
        axes = [torch.arange(n, device=device) for n in shape]
        idx = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
        out = [self._eval(self.points(idx[a:a + self.chunk], shape)) for a in range(0, idx.shape[0], self.chunk)]
        return torch.cat(out).to(dtype).reshape(shape)

    def band(self, shape, isovalue=0.0, dtype=torch.float32, background=None):
        """The narrow band of the field on a grid of `shape` (a BrickGrid whose values
        are differentiable with respect to the network's parameters)."""
        shape = tuple(int(n) for n in shape)
        device = next(self.net.parameters()).device
        nb = brick_dims(shape)
        iso = float(isovalue)
        st = self._steps(shape)
        # per brick, bounds of the field over its points and one grid step beyond (the
        # other ends of its edges): box [8 b - 1, 8 b + 8] in grid units
        with torch.no_grad():
            axes = [torch.arange(n, device=device) for n in nb]
            bidx = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
            lo_b, hi_b = [], []
            for a in range(0, bidx.shape[0], self.chunk):
                c = bidx[a:a + self.chunk]
                if self._lip is None and self.propagable():
                    l, h = self.bounds(self.points(c * B - 1, shape), self.points(c * B + B, shape))
                else:
                    if self._lip is None:
                        raise RuntimeError("this network has no interval bound: pass lipschitz=")
                    v = self._eval(self.points(c * B + 3.5, shape)).double()
                    reach = float(self._lip) * math.sqrt(sum((4.5 * s) ** 2 for s in st))
                    l, h = v - reach, v + reach
                lo_b.append(l)
                hi_b.append(h)
            lo_b, hi_b = torch.cat(lo_b), torch.cat(hi_b)
        # a margin for the rounding of evaluating the network in its dtype
        w = next(self.net.parameters())
        eps = (1e-5 if w.dtype != torch.float64 else 1e-12) * (abs(iso) + float(torch.maximum(lo_b.abs(),
                                                                                             hi_b.abs()).max()))
        above, below = lo_b > iso + eps, hi_b < iso - eps
        # the pad (iso + 1) meets the grid's faces: a brick there whose points may lie
        # below iso holds crossing edges to it
        edge = ((bidx == 0) | (bidx == torch.tensor(nb, device=device) - 1)).any(1)
        present = ~(above | below) | (edge & ~above)
        k = int(present.sum())
        index = torch.where(above, N.BRICK_OUTSIDE, N.BRICK_INSIDE).to(torch.int32)
        index[present] = torch.arange(k, dtype=torch.int32, device=device)
        bricks = bidx[present]
        lr = torch.arange(B, device=device)
        loc = torch.stack(torch.meshgrid(lr, lr, lr, indexing="ij"), -1).reshape(1, B ** 3, 3)
        hi = torch.tensor(shape, device=device) - 1
        # points beyond the grid's last row (bricks overhanging it) are never read:
        # they are evaluated at the clamped point
        pts_idx = torch.minimum(bricks[:, None, :] * B + loc, hi).reshape(-1, 3)
        per = max(1, self.chunk // (B ** 3)) * B ** 3
        chunks = []
        for a in range(0, pts_idx.shape[0], per):
            p = self.points(pts_idx[a:a + per], shape)
            if torch.is_grad_enabled() and any(q.requires_grad for q in self.net.parameters()):
                chunks.append(checkpoint(self._eval, p, use_reentrant=False))
            else:
                chunks.append(self._eval(p))
        values = (torch.cat(chunks).to(dtype) if chunks else torch.zeros(0, dtype=dtype, device=device))
        values = values.reshape(k, B, B, B)
        bg = float(background) if background is not None else 2.0 * abs(iso) + 1.0
        if not bg > abs(iso):
            raise RuntimeError("the background must exceed |isovalue| so that absent bricks keep their side")
        return BrickGrid(shape, index.reshape(nb), values, None, bg)


def extract_mlp(ex: N.Extractor, field: MLPField, shape, isovalue=0.0, normalize=True, return_quads=False,
                exact_grad=False):
    """The mesh of an MLP field on a grid of `shape` from its narrow band; the vertices
    are differentiable with respect to the network's parameters."""
    from .bricks import extract_bricks

    band = field.band(shape, isovalue, ex.dtype)
    return extract_bricks(ex, band, isovalue, normalize, return_quads, exact_grad)
