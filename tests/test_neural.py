"""MLP fields on the CPU: interval bounds that hold, a band that keeps every crossing
edge of the network's dense grid, and the fallback to a Lipschitz bound."""
import pytest
import torch
from torch import nn

from neural_nets import octahedron_net


def _crossings_inside(band, dense, iso=0.0):
    d, _ = band.dense()
    if not torch.equal(d >= iso, dense >= iso):
        return False
    present = d == dense
    side = dense >= iso
    for a in range(3):
        n = dense.shape[a]
        c = side.narrow(a, 1, n - 1) != side.narrow(a, 0, n - 1)
        if not (present.narrow(a, 1, n - 1)[c].all() and present.narrow(a, 0, n - 1)[c].all()):
            return False
    return True


def test_interval_bounds_hold():
    from diso_gb300 import MLPField

    f = MLPField(octahedron_net())
    g = torch.Generator().manual_seed(1)
    lo = torch.rand((500, 3), generator=g, dtype=torch.float64) * 1.8 - 1
    hi = lo + torch.rand((500, 3), generator=g, dtype=torch.float64) * 0.2
    bl, bh = f.bounds(lo, hi)
    assert (bl <= bh).all()
    for _ in range(20):
        p = lo + (hi - lo) * torch.rand((500, 3), generator=g, dtype=torch.float64)
        v = f._eval(p)
        assert (v >= bl - 1e-12).all() and (v <= bh + 1e-12).all()


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("shape,iso", [((61, 57, 66), 0.0), ((96, 96, 96), 0.1), ((40, 33, 70), -0.2)])
def test_band_keeps_every_crossing(dtype, shape, iso):
    from diso_gb300 import MLPField

    f = MLPField(octahedron_net(dtype))
    band = f.band(shape, iso, dtype)
    dense = f.dense(shape, dtype)
    assert 0 < band.count < band.index.numel()
    assert _crossings_inside(band, dense, iso)


def test_lipschitz_fallback_and_errors():
    from diso_gb300 import MLPField

    class Wrapped(nn.Module):  # not a Sequential: no interval propagation
        def __init__(self):
            super().__init__()
            self.inner = octahedron_net()

        def forward(self, p):
            return self.inner(p)

    with pytest.raises(RuntimeError, match="lipschitz"):
        MLPField(Wrapped()).band((32, 32, 32), 0.0, torch.float64)
    # a valid (loose) bound: every brick near the surface is kept, crossings inside
    f = MLPField(Wrapped(), lipschitz=20.0)
    band = f.band((48, 48, 48), 0.0, torch.float64)
    assert _crossings_inside(band, f.dense((48, 48, 48), torch.float64))
