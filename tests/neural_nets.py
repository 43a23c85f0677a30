"""Small MLP SDFs for the tests: an octahedron |x| + |y| + |z| - 0.8 written exactly as
a ReLU network (|t| = relu(t) + relu(-t)), plus a random ReLU branch scaled by 0.05,
so that the zero level set is a bent octahedron."""
import torch
from torch import nn


def octahedron_net(dtype=torch.float64, seed=0, width=32):
    g = torch.Generator().manual_seed(seed)
    net = nn.Sequential(nn.Linear(3, 6 + width), nn.ReLU(), nn.Linear(6 + width, 1 + width), nn.ReLU(),
                        nn.Linear(1 + width, 1))
    with torch.no_grad():
        for m in net:
            if isinstance(m, nn.Linear):
                m.weight.zero_()
                m.bias.zero_()
        net[0].weight[:3] = torch.eye(3)
        net[0].weight[3:6] = -torch.eye(3)
        net[0].weight[6:] = torch.randn((width, 3), generator=g) * 0.7
        net[0].bias[6:] = torch.randn(width, generator=g) * 0.2
        net[2].weight[0, :6] = 1.0
        net[2].weight[1:, 6:] = torch.randn((width, width), generator=g) * 0.3
        net[4].weight[0, 0] = 1.0
        net[4].weight[0, 1:] = torch.randn(width, generator=g) * 0.05
        net[4].bias.fill_(-0.8)
    return net.to(dtype)
