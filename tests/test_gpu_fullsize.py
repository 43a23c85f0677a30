"""The benchmark's own workload at full size: the 512^3 float32 grid (minimum of 16
seeded spheres plus N(0, 0.01) noise, deform U(-0.45, 0.45)), forward and backward,
against the float64 oracle (about a second per method on the host's cores), and
size-independent identities of the result: one DMC quad and one MC vertex per
crossing edge, bit-identical repeats."""
import numpy as np
import pytest
import torch

import bench
from helpers import assert_faces_equal, assert_grads_close, assert_verts_close, oracle_grad_rtol
from oracle import oracle as O

pytestmark = pytest.mark.gpu

N = 512


@pytest.fixture(scope="module")
def workload(cuda_device):
    sdf = bench.spheres_field(N, cuda_device)
    deform = bench.deform_field(N, cuda_device)
    return sdf, deform, sdf.cpu().numpy(), deform.cpu().numpy()


def _run(mod, sdf, deform, w=None, **kw):
    s = sdf.clone().requires_grad_(True)
    d = deform.clone().requires_grad_(True)
    v, f = mod(s, d, **kw)
    if w is None:
        w = bench.loss_weights(v.shape[0], sdf.device, torch.float32)
    (v * w).sum().backward()
    return v.detach(), f, s.grad, d.grad, w


@pytest.mark.parametrize("method", ["dmc", "mc"])
def test_benchmark_grid_against_oracle(cuda_device, workload, method):
    from diso_gb300 import DiffDMC, DiffMC

    sdf, deform, sn, dn = workload
    mod = DiffDMC(torch.float32) if method == "dmc" else DiffMC(torch.float32)
    kw = {"return_quads": True} if method == "dmc" else {}
    v, f, gs, gd, w = _run(mod, sdf, deform, **kw)
    case = dict(method=method, dtype="float32", iso=0.0, normalize=True, return_quads=True, shape=(N, N, N))
    m = O.DMC if method == "dmc" else O.MC
    v_ref, f_ref, _ = O.extract(m, sn, dn, 0.0, True, True, "float32")
    assert_verts_close(v.cpu().numpy(), v_ref, case)
    assert_faces_equal(f.cpu().numpy(), f_ref, case, v_ref)
    del v_ref, f_ref
    gs_ref, gd_ref = O.backward(m, sn, dn, w.cpu().numpy(), 0.0, True, "float32")
    rtol = oracle_grad_rtol("float32", (N, N, N))
    assert_grads_close(gs.cpu().numpy(), gs_ref, "float32", "grad_sdf", rtol)
    del gs_ref
    assert_grads_close(gd.cpu().numpy(), gd_ref, "float32", "grad_deform", rtol)
    # a second step through the same module (the single-call forward) repeats bit for bit
    v2, f2, gs2, gd2, _ = _run(mod, sdf, deform, w, **kw)
    assert torch.equal(v, v2) and torch.equal(f, f2) and torch.equal(gs, gs2) and torch.equal(gd, gd2)


def test_benchmark_grid_identities(cuda_device, workload):
    from diso_gb300 import DiffDMC, DiffMC

    sdf, deform, _, _ = workload
    with torch.no_grad():
        vm, fm = DiffMC(torch.float32)(sdf, deform)
        vq, q = DiffDMC(torch.float32)(sdf, deform, return_quads=True)
        vt, t = DiffDMC(torch.float32)(sdf, deform)
    # one MC vertex and one DMC quad per crossing edge; the split keeps every quad
    assert vm.shape[0] == q.shape[0] > 0
    assert t.shape[0] == 2 * q.shape[0] and torch.equal(vq, vt)
    # every index is in range and every dual vertex is a corner of some quad
    assert int(q.min()) >= 0 and int(q.max()) < vq.shape[0] and int(fm.max()) < vm.shape[0]
    used = torch.zeros(vq.shape[0], dtype=torch.bool, device=vq.device)
    used[q.reshape(-1)] = True
    assert bool(used.all())


def test_near_maximum_grid(cuda_device):
    # 860^3 (the C ABI accepts grids up to 3 (n+1)^3 < 2^31 cells, about 890^3): cell
    # records and segment indices beyond 2^31 entries of a row-major grid; MC and DMC
    # forwards agree on the crossing edges, every index is in range, every dual vertex
    # is used, and a repeat is bit-identical
    from diso_gb300 import DiffDMC, DiffMC

    n = 860
    sdf = bench.spheres_field(n, cuda_device)
    with torch.no_grad():
        vm, fm = DiffMC(torch.float32)(sdf)
        mod = DiffDMC(torch.float32)
        vq, q = mod(sdf, return_quads=True)
        vq2, q2 = mod(sdf, return_quads=True)
    assert vm.shape[0] == q.shape[0] > 0
    assert int(q.min()) >= 0 and int(q.max()) < vq.shape[0] and int(fm.max()) < vm.shape[0]
    used = torch.zeros(vq.shape[0], dtype=torch.bool, device=vq.device)
    used[q.reshape(-1)] = True
    assert bool(used.all())
    assert torch.equal(vq, vq2) and torch.equal(q, q2)
    assert float(vq.min()) >= -0.01 and float(vq.max()) <= 1.01  # normalised to the grid
