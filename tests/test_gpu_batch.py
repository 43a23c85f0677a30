"""Batched extraction (one launch per phase for many grids of uneven size):
every grid's mesh and gradients equal the single-grid API's, eagerly and under
CUDA-graph replay."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _fields(shapes, seed, dtype=np.float32):
    rng = np.random.default_rng(seed)
    out = []
    for k, sh in enumerate(shapes):
        axes = [np.linspace(-1, 1, n) for n in sh]
        X, Y, Z = np.meshgrid(*axes, indexing="ij")
        if k % 3 == 2:
            s = rng.uniform(-1, 1, sh)
        else:
            r = rng.uniform(0.3, 0.7)
            s = np.sqrt(X * X + Y * Y + Z * Z) - r + 0.02 * rng.standard_normal(sh)
        out.append(s.astype(dtype))
    return out


SHAPES = [(40, 33, 35), (17, 64, 20), (9, 9, 9), (64, 64, 64), (3, 50, 2), (33, 31, 70)]


@pytest.mark.parametrize("method,rq", [("mc", False), ("dmc", True), ("dmc", False)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_batch_matches_single(cuda_device, method, rq, dtype):
    from diso_gb300 import DiffDMC, DiffDMCBatch, DiffMC, DiffMCBatch

    npdt = np.float32 if dtype == torch.float32 else np.float64
    fields = _fields(SHAPES, 3, npdt)
    rng = np.random.default_rng(4)
    defs = [rng.uniform(-0.3, 0.3, f.shape + (3,)).astype(npdt) for f in fields]
    isos = [0.0, 0.05, -0.02, 0.0, 0.1, 0.0]
    single = DiffMC(dtype) if method == "mc" else DiffDMC(dtype)
    batch = DiffMCBatch(dtype) if method == "mc" else DiffDMCBatch(dtype)
    s_b = [torch.tensor(f, device=cuda_device, requires_grad=True) for f in fields]
    d_b = [torch.tensor(d, device=cuda_device, requires_grad=True) for d in defs]
    if method == "mc":
        outs = batch(s_b, d_b, isovalue=isos)
    else:
        outs = batch(s_b, d_b, isovalue=isos, return_quads=rq)
    loss = 0
    ws = []
    for (v, f), k in zip(outs, range(len(outs))):
        w = torch.randn(v.shape, dtype=dtype, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(k))
        ws.append(w)
        loss = loss + (v * w).sum()
    loss.backward()
    for i, f in enumerate(fields):
        s = torch.tensor(f, device=cuda_device, requires_grad=True)
        d = torch.tensor(defs[i], device=cuda_device, requires_grad=True)
        v, fc = single(s, d, isovalue=isos[i]) if method == "mc" else single(s, d, isovalue=isos[i], return_quads=rq)
        vb, fb = outs[i]
        assert fb.dtype == fc.dtype and torch.equal(fb, fc), f"grid {i}: faces differ"
        assert torch.equal(vb, v), f"grid {i}: vertices differ"
        if not v.requires_grad:  # the empty-surface guard fired: no mesh, no gradient
            assert v.shape[0] == 0 and not s_b[i].grad.any() and not d_b[i].grad.any()
            continue
        (v * ws[i]).sum().backward()
        assert torch.equal(s_b[i].grad, s.grad), f"grid {i}: grad_sdf differs"
        assert torch.equal(d_b[i].grad, d.grad), f"grid {i}: grad_deform differs"


@pytest.mark.parametrize("method", [0, 1])
def test_batch_plan_graph_replay(cuda_device, method):
    from diso_gb300 import BatchPlan
    from diso_gb300 import _native as N

    shapes = [(48, 40, 33), (20, 20, 20), (64, 30, 50), (11, 70, 9)]
    plan = BatchPlan(method, torch.float32, shapes, deform=True)
    rng = np.random.default_rng(7)
    fields = _fields(shapes, 5)
    for i, f in enumerate(fields):
        plan.sdf[i].copy_(torch.tensor(f))
        plan.deform[i].copy_(torch.tensor(rng.uniform(-0.3, 0.3, f.shape + (3,)).astype(np.float32)))
    nv, nf = plan.size_outputs()
    plan.grad_verts[:nv].normal_(generator=torch.Generator(cuda_device).manual_seed(1))
    plan.run()  # eager
    eager = [(v.clone(), f.clone()) for v, f in plan.meshes()]
    eager_g = [g.clone() for g in plan.grad_sdf] + [g.clone() for g in plan.grad_deform]
    for _ in range(3):
        plan.replay()
    torch.cuda.synchronize()
    for (v, f), (ve, fe) in zip(plan.meshes(), eager):
        assert torch.equal(v, ve) and torch.equal(f, fe)
    for g, ge in zip(list(plan.grad_sdf) + list(plan.grad_deform), eager_g):
        assert torch.equal(g, ge)
    # change the inputs in place: the same graph now extracts the new fields
    fields2 = _fields(shapes, 9)
    for i, f in enumerate(fields2):
        plan.sdf[i].copy_(torch.tensor(f))
    plan.replay()
    meshes = plan.meshes()
    ex = N.Extractor(method, torch.float32)
    from diso_gb300.extraction import extract
    for i, f in enumerate(fields2):
        v, fc = extract(ex, torch.tensor(f, device=cuda_device), plan.deform[i], 0.0, True, True)
        assert torch.equal(meshes[i][1], fc) and torch.equal(meshes[i][0], v)


@pytest.mark.parametrize("method,rq", [("mc", False), ("dmc", True)])
def test_uneven_batch_at_full_size(cuda_device, method, rq):
    """The batched workload itself: 64 grids, N log-uniform in [32, 256] (seeded),
    spheres and rounded boxes with N(0, 0.02) noise, deform U(-0.3, 0.3) (about 10^8
    cells in one flattened queue); every grid's mesh and gradients equal the
    single-grid module's bit for bit."""
    import bench
    from diso_gb300 import DiffDMC, DiffDMCBatch, DiffMC, DiffMCBatch

    sdfs, defs = bench.uneven_batch(64, device=cuda_device)
    assert sum(s.numel() for s in sdfs) > 5e7
    batch = DiffMCBatch(torch.float32) if method == "mc" else DiffDMCBatch(torch.float32)
    single = DiffMC(torch.float32) if method == "mc" else DiffDMC(torch.float32)
    kw = {} if method == "mc" else {"return_quads": rq}
    s_b = [s.clone().requires_grad_(True) for s in sdfs]
    d_b = [d.clone().requires_grad_(True) for d in defs]
    outs = batch(s_b, d_b, **kw)
    ws = [torch.randn(v.shape, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(k))
          for k, (v, _) in enumerate(outs)]
    sum((v * w).sum() for (v, _), w in zip(outs, ws)).backward()
    for i in range(len(sdfs)):
        s = sdfs[i].clone().requires_grad_(True)
        d = defs[i].clone().requires_grad_(True)
        v, f = single(s, d, **kw)
        assert torch.equal(outs[i][1], f) and torch.equal(outs[i][0], v), f"grid {i}: mesh differs"
        (v * ws[i]).sum().backward()
        assert torch.equal(s_b[i].grad, s.grad) and torch.equal(d_b[i].grad, d.grad), f"grid {i}: gradients differ"
