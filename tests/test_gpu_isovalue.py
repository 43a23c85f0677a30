"""dL/d(isovalue), which the reference does not give (its isovalue is a plain
scalar): an isovalue passed as a tensor that requires grad receives minus the sum of
dL/dsdf, reduced natively over the point tiles near the surface.  Checked against
central differences of the extraction itself (float64), the oracle's backward,
the sum of the returned dL/dsdf, a whole-grid reduction, and per grid in batches."""
import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _field(n, kind, seed, npdt):
    rng = np.random.default_rng(seed)
    a = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    # the plane crosses the grid's faces: edges to the pad carry vertices too
    base = np.sqrt(X * X + Y * Y + Z * Z) - 0.5 if kind == "sphere" else 0.6 * X + 0.3 * Y - 0.2 * Z - 0.1
    sdf = (base + 0.03 * rng.standard_normal((n, n, n))).astype(npdt)
    deform = rng.uniform(-0.3, 0.3, (n, n, n, 3)).astype(npdt)
    return sdf, deform


def _module(method, dtype, exact=True):
    from diso_gb300 import DiffDMC, DiffMC

    return DiffMC(dtype) if method == "mc" else DiffDMC(dtype, exact_grad=exact)


def _loss_weights(n, dtype, dev, seed=0):
    return torch.randn((n, 3), dtype=dtype, device=dev, generator=torch.Generator(dev).manual_seed(seed))


@pytest.mark.parametrize("method", ["mc", "dmc"])
@pytest.mark.parametrize("kind", ["sphere", "plane"])
def test_isovalue_grad_finite_differences(cuda_device, method, kind):
    sdf_np, def_np = _field(24, kind, 7, np.float64)
    sdf = torch.tensor(sdf_np, device=cuda_device)
    deform = torch.tensor(def_np, device=cuda_device)
    mod = _module(method, torch.float64)
    iso0, h = 0.02, 1e-6
    iso = torch.tensor(iso0, dtype=torch.float64, requires_grad=True)
    v, f = mod(sdf, deform, iso)
    w = _loss_weights(v.shape[0], torch.float64, cuda_device)
    (v * w).sum().backward()
    g = float(iso.grad)
    assert iso.grad.dtype == torch.float64 and iso.grad.shape == () and iso.grad.device.type == "cpu"
    with torch.no_grad():
        vp, fp = mod(sdf, deform, iso0 + h)
        vm, fm = mod(sdf, deform, iso0 - h)
    assert torch.equal(fp, f) and torch.equal(fm, f)  # the same crossings at both ends
    fd = float(((vp * w).sum() - (vm * w).sum()) / (2 * h))
    assert abs(fd - g) <= 1e-6 * max(1.0, abs(fd)), (fd, g)
    # the oracle's backward (exact derivative) gives the same sum
    m = O.MC if method == "mc" else O.DMC
    gs_ref, _ = O.backward(m, sdf_np, def_np, w.cpu().numpy(), iso0, True, "float64", exact=True)
    assert abs(g + gs_ref.sum()) <= 1e-9 * max(1.0, np.abs(gs_ref).sum()), (g, -gs_ref.sum())


@pytest.mark.parametrize("method,exact", [("mc", False), ("dmc", False), ("dmc", True)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_isovalue_grad_is_minus_sdf_grad_sum(cuda_device, method, exact, dtype):
    npdt = np.float32 if dtype == torch.float32 else np.float64
    sdf_np, def_np = _field(48, "sphere", 8, npdt)
    s = torch.tensor(sdf_np, device=cuda_device, requires_grad=True)
    d = torch.tensor(def_np, device=cuda_device, requires_grad=True)
    iso = torch.tensor(0.01, dtype=dtype, device=cuda_device, requires_grad=True)
    mod = _module(method, dtype, exact)
    v, f = mod(s, d, iso)
    w = _loss_weights(v.shape[0], dtype, cuda_device, 1)
    (v * w).sum().backward()
    assert iso.grad.dtype == dtype and iso.grad.device == iso.device and iso.grad.shape == ()
    ref = -s.grad.double().sum()
    tol = (1e-6 if dtype == torch.float32 else 1e-12) * float(s.grad.double().abs().sum())
    assert abs(float(iso.grad) - float(ref)) <= tol, (float(iso.grad), float(ref))
    # repeats bit for bit; an isovalue alone asks for no gradient of the grid
    g1 = iso.grad.clone()
    s2 = s.detach().clone()
    iso2 = iso.detach().clone().requires_grad_(True)
    v2, _ = mod(s2, d.detach(), iso2)
    (v2 * w).sum().backward()
    assert torch.equal(iso2.grad, g1) and s2.grad is None


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
def test_isovalue_grad_near_surface_tiles_equal_whole_grid(cuda_device, dtype):
    # the reduction that reads only the point tiles near the surface (with the
    # forward's record) equals the one over the whole grid
    from diso_gb300 import _native as N
    from diso_gb300.extraction import extract

    npdt = np.float32 if dtype == torch.float32 else np.float64
    sdf_np, def_np = _field(160, "sphere", 9, npdt)
    s = torch.tensor(sdf_np, device=cuda_device, requires_grad=True)
    ex = N.Extractor(N.DMC, dtype)
    v, f = extract(ex, s, torch.tensor(def_np, device=cuda_device), 0.0, True, True)
    (v * _loss_weights(v.shape[0], dtype, cuda_device, 2)).sum().backward()
    whole = ex.isovalue_grad(s.grad)
    g = s.grad.contiguous()
    seg = torch.empty(N.Extractor.segment_slots(g.shape), dtype=torch.int64, device=cuda_device)
    ex.count(s.detach(), *N.iso_values(0.0, dtype), seg)
    near = ex.isovalue_grad(g, seg)
    assert torch.equal(near, whole)
    tol = (1e-6 if dtype == torch.float32 else 1e-12) * float(g.double().abs().sum())
    assert abs(float(whole) + float(g.double().sum())) <= tol


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_batch_isovalue_grads_per_grid(cuda_device, method):
    from diso_gb300 import DiffDMCBatch, DiffMCBatch

    dtype = torch.float32
    shapes = [(40, 33, 35), (17, 64, 20), (64, 64, 64)]
    rng = np.random.default_rng(10)
    grids, isos0 = [], [0.0, 0.05, -0.02]
    for sh in shapes:
        X, Y, Z = np.meshgrid(*[np.linspace(-1, 1, n) for n in sh], indexing="ij")
        grids.append((np.sqrt(X * X + Y * Y + Z * Z) - rng.uniform(0.3, 0.7)
                      + 0.02 * rng.standard_normal(sh)).astype(np.float32))
    batch = DiffMCBatch(dtype) if method == "mc" else DiffDMCBatch(dtype, exact_grad=True)
    single = _module(method, dtype)
    sb = [torch.tensor(g, device=cuda_device) for g in grids]
    isos = [torch.tensor(x, device=cuda_device, requires_grad=True) for x in isos0]
    outs = batch(sb, None, isovalue=isos)
    ws = [_loss_weights(v.shape[0], dtype, cuda_device, 20 + k) for k, (v, _) in enumerate(outs)]
    sum((v * w).sum() for (v, _), w in zip(outs, ws)).backward()
    for i in range(len(grids)):
        iso = torch.tensor(isos0[i], device=cuda_device, requires_grad=True)
        v, _ = single(sb[i], None, iso)
        (v * ws[i]).sum().backward()
        assert torch.equal(isos[i].grad, iso.grad), (i, float(isos[i].grad), float(iso.grad))
    # one isovalue tensor shared by every grid: the sum of the grids' gradients
    shared = torch.tensor(0.0, device=cuda_device, requires_grad=True)
    outs = batch(sb, None, isovalue=shared)
    ws = [_loss_weights(v.shape[0], dtype, cuda_device, 30 + k) for k, (v, _) in enumerate(outs)]
    sum((v * w).sum() for (v, _), w in zip(outs, ws)).backward()
    parts = []
    for i in range(len(grids)):
        iso = torch.tensor(0.0, device=cuda_device, requires_grad=True)
        v, _ = single(sb[i], None, iso)
        (v * ws[i]).sum().backward()
        parts.append(float(iso.grad))
    assert abs(float(shared.grad) - sum(parts)) <= 1e-6 * max(1.0, sum(abs(p) for p in parts))
