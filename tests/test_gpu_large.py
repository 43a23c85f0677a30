"""Dense grids past the worst-case 32-bit limit (3 crossings per cell below 2^31: about
890^3).  A 1024^3 sphere through the dense path equals the same grid cut to a narrow
band (both paths are tied to the oracle at smaller sizes): vertices and faces bit for
bit, gradients at the bricks' points.  A 1024^3 grid whose every edge crosses (3.2 G
crossings) is rejected after its count, and the extractor works afterwards."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def _sphere(n, device, r=0.6):
    a = torch.linspace(-1, 1, n, device=device)
    return torch.sqrt(a.view(-1, 1, 1) ** 2 + a.view(1, -1, 1) ** 2 + a.view(1, 1, -1) ** 2) - r


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_dense_1024_equals_its_band(cuda_device, method):
    from diso_gb300 import BrickGrid, DiffDMC, DiffMC
    from diso_gb300.bricks import _to_bricks, brick_dims

    n = 1024
    sdf = _sphere(n, cuda_device)
    mod = DiffMC(torch.float32) if method == "mc" else DiffDMC(torch.float32)
    kw = {} if method == "mc" else {"return_quads": True}
    s = sdf.clone().requires_grad_(True)
    v, f = mod(s, **kw)
    assert v.shape[0] > 1_000_000
    w = torch.randn(v.shape, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(1))
    (v * w).sum().backward()
    band = BrickGrid.from_dense(sdf, 0.0)
    del sdf
    band.values.requires_grad_(True)
    v2, f2 = mod.forward_bricks(band, **kw)
    assert torch.equal(v.detach(), v2.detach()) and torch.equal(f, f2)
    (v2 * w).sum().backward()
    sel = torch.nonzero(band.index.reshape(-1) >= 0).flatten()
    assert torch.equal(band.values.grad, _to_bricks(s.grad, brick_dims((n, n, n)), 0.0)[sel])


def test_overflowing_counts_are_rejected(cuda_device):
    from diso_gb300 import DiffMC

    n = 1024
    i = torch.arange(n, device=cuda_device)
    # a 3-d checkerboard: every edge crosses, 3 crossings per cell
    sdf = (((i.view(-1, 1, 1) + i.view(1, -1, 1) + i.view(1, 1, -1)) % 2) * 2 - 1).to(torch.float32)
    mod = DiffMC(torch.float32)
    with pytest.raises(RuntimeError, match="too many crossings"):
        mod(sdf)
    del sdf
    v, f = mod(_sphere(64, cuda_device))
    assert v.shape[0] > 1000 and f.shape[0] > 1000
