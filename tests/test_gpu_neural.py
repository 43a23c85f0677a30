"""MLP fields on the GPU: the mesh from the network's narrow band (DiffMC /
DiffDMC.forward_mlp) against the dense path on the network's values over the whole
grid, and the gradients of the network's parameters through both paths."""
import pytest
import torch

from neural_nets import octahedron_net

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("method,rq", [("mc", False), ("dmc", True), ("dmc", False)])
@pytest.mark.parametrize("shape,iso", [((96, 96, 96), 0.0), ((71, 64, 90), 0.1)])
def test_mlp_band_matches_dense(cuda_device, method, rq, shape, iso):
    from diso_gb300 import DiffDMC, DiffMC, MLPField

    dt = torch.float64
    net = octahedron_net(dt).to(cuda_device)
    field = MLPField(net)
    mod = DiffMC(dt) if method == "mc" else DiffDMC(dt)
    kw = {} if method == "mc" else {"return_quads": rq}
    v, f = mod.forward_mlp(field, shape, isovalue=iso, **kw)
    # the dense path on the network's values over the whole grid
    dense = field.dense(shape, dt)
    v2, f2 = mod(dense, isovalue=iso, **kw)
    assert v.shape[0] > 1000
    assert torch.equal(f, f2), "faces differ from the dense path"
    # a point's value may round differently inside another batch of the network
    assert (v - v2).abs().max().item() < 1e-9
    w = torch.randn(v.shape, dtype=dt, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(3))
    (v * w).sum().backward()
    g_band = [p.grad.clone() for p in net.parameters()]
    net.zero_grad()
    dense = field.dense(shape, dt)  # now with the graph to the parameters
    v2, _ = mod(dense, isovalue=iso, **kw)
    (v2 * w).sum().backward()
    for a, b in zip(g_band, (p.grad for p in net.parameters())):
        assert (a - b).abs().max().item() <= 1e-9 * max(1.0, b.abs().max().item())


def test_mlp_band_is_a_fraction_of_the_grid(cuda_device):
    from diso_gb300 import DiffDMC, MLPField

    net = octahedron_net(torch.float32).to(cuda_device)
    field = MLPField(net)
    band = field.band((512, 512, 512), 0.0, torch.float32)
    assert band.count < 0.15 * band.index.numel(), (band.count, band.index.numel())
    v, q = DiffDMC(torch.float32).forward_bricks(band, return_quads=True)
    assert v.shape[0] > 100_000 and q.shape[0] > 100_000, (v.shape, q.shape)
    # every vertex lies near the bent octahedron: |x| + |y| + |z| within 0.8 +- 0.2 on
    # [-1, 1]^3 (normalised vertices are in [0, 1]^3)
    l1 = (2 * v.detach() - 1).abs().sum(1)
    assert l1.min().item() > 0.6 and l1.max().item() < 1.0, (l1.min().item(), l1.max().item())
