"""recompute=True: the forward keeps no edge record and no gradient buffers, only
its segment record (the reference keeps nothing and its backward re-runs the
forward, diso/__init__.py:32, 86); the backward recomputes the crossing lists per
point tile in one fused pass (diso_backward_recompute).  Outputs and gradients
equal the default mode's bit for bit (also where a tile's window holds too many
crossing edges for the shared-memory cache, on dense random fields), and the
forward holds less device memory."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _inputs(n, dtype, dev, seed):
    rng = np.random.default_rng(seed)
    a = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    npdt = np.float32 if dtype == torch.float32 else np.float64
    sdf = (np.sqrt(X * X + Y * Y + Z * Z) - 0.55 + 0.03 * rng.standard_normal((n, n, n))).astype(npdt)
    deform = rng.uniform(-0.3, 0.3, (n, n, n, 3)).astype(npdt)
    return torch.tensor(sdf, device=dev), torch.tensor(deform, device=dev)


def _module(method, dtype, recompute):
    from diso_gb300 import DiffDMC, DiffMC

    return DiffMC(dtype, recompute=recompute) if method == "mc" else DiffDMC(dtype, recompute=recompute)


def _step(mod, sdf, deform, kw, iso=0.0):
    s = sdf.clone().requires_grad_(True)
    d = deform.clone().requires_grad_(True) if deform is not None else None
    v, f = mod(s, d, iso, **kw)
    w = torch.randn(v.shape, dtype=v.dtype, device=v.device, generator=torch.Generator(v.device).manual_seed(3))
    (v * w).sum().backward()
    return v.detach(), f, s.grad, d.grad if d is not None else None


@pytest.mark.parametrize("method,kw", [("mc", {}), ("dmc", {"return_quads": True}), ("dmc", {})])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("with_deform", [True, False])
def test_recompute_equals_stored(cuda_device, method, kw, dtype, with_deform):
    sdf, deform = _inputs(40, dtype, cuda_device, 1)
    deform = deform if with_deform else None
    for iso in (0.0, 0.02):
        a = _step(_module(method, dtype, False), sdf, deform, kw, iso)
        b = _step(_module(method, dtype, True), sdf, deform, kw, iso)
        for x, y in zip(a, b):
            assert (x is None and y is None) or torch.equal(x, y)


def _dense(shape, dtype, dev, seed):
    rng = np.random.default_rng(seed)
    npdt = np.float32 if dtype == torch.float32 else np.float64
    sdf = rng.uniform(-1, 1, shape).astype(npdt)
    deform = rng.uniform(-0.45, 0.45, shape + (3,)).astype(npdt)
    return torch.tensor(sdf, device=dev), torch.tensor(deform, device=dev)


@pytest.mark.parametrize("method,kw,exact", [("mc", {}, False), ("dmc", {"return_quads": True}, False),
                                             ("dmc", {"return_quads": True}, True)])
@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("shape,field", [((37, 50, 70), "dense"), ((65, 33, 97), "sphere"),
                                         ((96, 96, 96), "dense"), ((72, 40, 200), "sphere")])
def test_fused_backward_equals_stored(cuda_device, method, kw, exact, dtype, shape, field):
    """Dense U(-1, 1) fields put thousands of crossing edges in a tile's window (the
    uncached path); odd sizes leave partial tiles on every axis and rows that are no
    multiple of 16 bytes (the zeros by a kernel on the second stream); rows of whole
    16-byte units get their zeros as bulk copies from inside the fused pass, the long
    z extent of (72, 40, 200) with runs of idle tiles; exact_grad takes each patch's
    own gradient."""
    from diso_gb300 import DiffDMC, DiffMC

    if field == "dense":
        sdf, deform = _dense(shape, dtype, cuda_device, 5)
    else:
        rng = np.random.default_rng(6)
        X, Y, Z = np.meshgrid(*[np.linspace(-1, 1, n) for n in shape], indexing="ij")
        npdt = np.float32 if dtype == torch.float32 else np.float64
        sdf = torch.tensor((np.sqrt(X * X + Y * Y + Z * Z) - 0.55 + 0.03 * rng.standard_normal(shape)).astype(npdt),
                           device=cuda_device)
        deform = torch.tensor(rng.uniform(-0.3, 0.3, shape + (3,)).astype(npdt), device=cuda_device)
    res = []
    for recompute in (False, True):
        mod = (DiffMC(dtype, recompute=recompute) if method == "mc"
               else DiffDMC(dtype, recompute=recompute, exact_grad=exact))
        for normalize in (True, False):
            s = sdf.clone().requires_grad_(True)
            d = deform.clone().requires_grad_(True)
            v, f = mod(s, d, 0.0, normalize=normalize, **kw)
            w = torch.randn(v.shape, dtype=v.dtype, device=v.device,
                            generator=torch.Generator(v.device).manual_seed(7))
            (v * w).sum().backward()
            res.append((v.detach(), f, s.grad, d.grad))
    for x, y in zip(res[:2], res[2:]):
        for a, b in zip(x, y):
            assert torch.equal(a, b)


def test_fused_backward_repeats_bit_for_bit(cuda_device):
    from diso_gb300 import DiffDMC

    sdf, deform = _dense((48, 48, 48), torch.float32, cuda_device, 8)
    mod = DiffDMC(torch.float32, recompute=True)
    out = []
    for _ in range(3):
        s = sdf.clone().requires_grad_(True)
        d = deform.clone().requires_grad_(True)
        v, _ = mod(s, d, return_quads=True)
        (v * v).sum().backward()
        out.append((s.grad, d.grad))
    for a, b in out[1:]:
        assert torch.equal(a, out[0][0]) and torch.equal(b, out[0][1])


def test_recompute_isovalue_grad(cuda_device):
    sdf, deform = _inputs(32, torch.float64, cuda_device, 2)
    out = []
    for recompute in (False, True):
        iso = torch.tensor(0.01, dtype=torch.float64, device=cuda_device, requires_grad=True)
        v, _ = _module("dmc", torch.float64, recompute)(sdf, deform, iso)
        (v * v).sum().backward()
        out.append(iso.grad)
    assert torch.equal(out[0], out[1])


def test_recompute_holds_less_memory(cuda_device):
    n = 96
    sdf, deform = _inputs(n, torch.float32, cuda_device, 3)
    held = {}
    for recompute in (False, True):
        mod = _module("dmc", torch.float32, recompute)
        with torch.no_grad():
            mod(sdf, deform)  # the size hint for this shape
        s = sdf.clone().requires_grad_(True)
        d = deform.clone().requires_grad_(True)
        torch.cuda.synchronize()
        m0 = torch.cuda.memory_allocated(cuda_device)
        v, f = mod(s, d, return_quads=True)
        torch.cuda.synchronize()
        held[recompute] = torch.cuda.memory_allocated(cuda_device) - m0
        v.sum().backward()
        del v, f, s, d
    # the default forward holds the gradient buffers (4 n^3 floats) and the edge record
    assert held[True] + 4 * n ** 3 * 4 <= held[False], held


def test_recompute_detects_a_changed_grid(cuda_device):
    sdf, _ = _inputs(24, torch.float32, cuda_device, 4)
    s = sdf.clone().requires_grad_(True)
    v, _ = _module("mc", torch.float32, True)(s)
    with torch.no_grad():
        s.add_(0.5)  # in place, after the forward: autograd's version check refuses the backward
    with pytest.raises(RuntimeError):
        v.sum().backward()


@pytest.mark.parametrize("method,kw", [("mc", {}), ("dmc", {"return_quads": True}), ("dmc", {})])
@pytest.mark.parametrize("recompute", [False, True])
def test_interleaved_forwards_before_one_backward(cuda_device, method, kw, recompute):
    """Forward of grid A, forward of grid B on the same module, then one backward of
    lossA + lossB: the case the reference re-runs its forward in backward for
    (diso/__init__.py:32, 86).  Each grid's gradients equal those of a module that
    saw only that grid."""
    sdf_a, def_a = _inputs(40, torch.float32, cuda_device, 11)
    sdf_b, def_b = _dense((33, 45, 38), torch.float32, cuda_device, 12)
    mod = _module(method, torch.float32, recompute)
    sa, da = sdf_a.clone().requires_grad_(True), def_a.clone().requires_grad_(True)
    sb, db = sdf_b.clone().requires_grad_(True), def_b.clone().requires_grad_(True)
    va, fa = mod(sa, da, **kw)
    vb, fb = mod(sb, db, **kw)
    wa = torch.randn(va.shape, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(1))
    wb = torch.randn(vb.shape, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(2))
    ((va * wa).sum() + (vb * wb).sum()).backward()
    for s_in, d_in, w, v0, f0, s_g, d_g in ((sdf_a, def_a, wa, va, fa, sa, da), (sdf_b, def_b, wb, vb, fb, sb, db)):
        s = s_in.clone().requires_grad_(True)
        d = d_in.clone().requires_grad_(True)
        v, f = _module(method, torch.float32, recompute)(s, d, **kw)
        assert torch.equal(v, v0.detach()) and torch.equal(f, f0)
        (v * w).sum().backward()
        assert torch.equal(s.grad, s_g.grad) and torch.equal(d.grad, d_g.grad)
