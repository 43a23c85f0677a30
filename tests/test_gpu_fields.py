"""The fused forward of an evaluated field (DiffMC / DiffDMC.forward_field over
diso_forward_field) against the dense forward on the same field's grid
(field.materialize), which the other parity tests tie to the reference: vertices and
faces must be identical, bit for bit, including where the count classified whole
chunks without evaluating them."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

DT = {"float32": torch.float32, "float64": torch.float64}


def _field(kind, device, dtype):
    from diso_gb300 import SphereUnion

    rng = np.random.default_rng(7)
    if kind == "example":  # the reference example's sphere and bounding box (test/example.py:20-53)
        m = 0.5 + 1 / 64
        return SphereUnion(torch.zeros(1, 3, device=device, dtype=dtype), torch.full((1,), 0.5, device=device,
                                                                                        dtype=dtype), (-m,) * 3, (m,) * 3)
    if kind == "spheres":
        c = rng.uniform(-0.8, 0.8, (16, 3))
        r = rng.uniform(0.05, 0.3, 16)
    elif kind == "faces":  # spheres through the grid's faces
        c = np.array([[1.0, 0.0, 0.0], [-0.2, -1.0, 0.3], [0.1, 0.2, 0.95]])
        r = np.array([0.5, 0.4, 0.3])
    elif kind == "inside":  # one sphere holding the whole grid: every value below iso, so the guard
        c, r = np.zeros((1, 3)), np.array([3.0])
    elif kind == "far":  # no surface: the empty-surface guard
        c, r = np.array([[5.0, 5.0, 5.0]]), np.array([0.5])
    elif kind == "small":  # few small spheres on a large grid: most chunks classified whole
        c = rng.uniform(-0.6, 0.6, (4, 3))
        r = rng.uniform(0.05, 0.12, 4)
    return SphereUnion(torch.tensor(c, device=device, dtype=dtype), torch.tensor(r, device=device, dtype=dtype))


CASES = [
    # (field, shape, iso, normalize)
    ("example", (64, 64, 64), 0.0, True),
    ("spheres", (96, 80, 112), 0.0, True),
    ("faces", (70, 65, 33), 0.0, True),
    ("spheres", (57, 40, 77), 0.1, False),
    ("inside", (40, 37, 50), 0.0, True),
    ("far", (48, 48, 48), 0.0, True),
    ("small", (160, 160, 160), 0.0, True),
]


@pytest.mark.parametrize("method", ["mc", "dmc"])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("kind,shape,iso,normalize", CASES)
def test_fused_field_matches_dense(cuda_device, method, dtype, kind, shape, iso, normalize):
    from diso_gb300 import DiffDMC, DiffMC

    dt = DT[dtype]
    field = _field(kind, cuda_device, dt)
    grid = field.materialize(shape, dt)
    mod = DiffMC(dt) if method == "mc" else DiffDMC(dt)
    variants = [{}] if method == "mc" else [{"return_quads": True}, {"return_quads": False}]
    for kw in variants:
        for _ in range(2):  # the second call uses the capacities the first one learned
            v, f = mod.forward_field(field, shape, isovalue=iso, normalize=normalize, **kw)
            with torch.no_grad():
                vd, fd = mod(grid, isovalue=iso, normalize=normalize, **kw)
            assert v.shape == vd.shape and f.shape == fd.shape and f.dtype == fd.dtype, (kw, v.shape, vd.shape)
            assert torch.equal(v, vd) and torch.equal(f, fd), kw
    if kind in ("far", "inside"):  # the empty-surface guard (all values above / below iso)
        assert v.shape[0] == 0 and f.dtype == torch.int32
    else:
        assert v.shape[0] > 0


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_materialize_matches_the_field_definition(cuda_device, dtype):
    # value(p) = min_k (|p - c_k| - r_k) at p = lo + (hi - lo) * i / (n - 1), against a
    # float64 numpy evaluation (within rounding: the device contracts lo + step * i)
    dt = DT[dtype]
    field = _field("spheres", cuda_device, dt)
    shape = (23, 17, 31)
    got = field.materialize(shape, dt).cpu().numpy().astype(np.float64)
    sph = field.spheres.cpu().numpy().astype(np.float64)
    axes = [np.asarray(field.lo[a]) + (field.hi[a] - field.lo[a]) / (shape[a] - 1) * np.arange(shape[a])
            for a in range(3)]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    ref = np.full(shape, np.inf)
    for cx, cy, cz, r in sph:
        ref = np.minimum(ref, np.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) - r)
    assert np.abs(got - ref).max() <= (1e-5 if dtype == "float32" else 1e-12)


@pytest.mark.parametrize("method,rq", [("mc", False), ("dmc", True), ("dmc", False)])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("kind,shape,iso,normalize", [("spheres", (96, 80, 112), 0.0, True),
                                                      ("faces", (70, 65, 33), 0.0, True),
                                                      ("spheres", (57, 40, 77), 0.1, False)])
def test_fused_field_matches_oracle(cuda_device, method, rq, dtype, kind, shape, iso, normalize):
    """The fused forward against the float64 oracle on the field's grid, so that the
    evaluated-field path is tied to the reference's algorithm directly, not only
    through the dense CUDA path."""
    from diso_gb300 import DiffDMC, DiffMC
    from helpers import assert_faces_equal, assert_verts_close
    from oracle import oracle as O

    dt = DT[dtype]
    field = _field(kind, cuda_device, dt)
    grid = field.materialize(shape, dt).cpu().numpy()
    if method == "mc":
        v, f = DiffMC(dt).forward_field(field, shape, iso, normalize)
    else:
        v, f = DiffDMC(dt).forward_field(field, shape, iso, rq, normalize)
    m = O.MC if method == "mc" else O.DMC
    v_ref, f_ref, _ = O.extract(m, grid, None, iso, normalize, rq, dtype)
    case = dict(method=method, dtype=dtype, iso=iso, normalize=normalize, return_quads=rq, shape=shape)
    assert_verts_close(v.cpu().numpy(), v_ref, case)
    assert_faces_equal(f.cpu().numpy(), f_ref, case, v_ref)


def _grad_field(dev, dt, K=4, seed=3):
    from diso_gb300 import SphereUnion

    rng = np.random.default_rng(seed)
    c = torch.tensor(rng.uniform(-0.5, 0.5, (K, 3)), device=dev, dtype=dt, requires_grad=True)
    r = torch.tensor(rng.uniform(0.2, 0.45, K), device=dev, dtype=dt, requires_grad=True)
    return c, r, SphereUnion(c, r)


def _chain_rule(field, shape, gsdf):
    """dL/d(centres, radii) from a dense dL/dsdf: each point's gradient to the sphere
    attaining the minimum there (float64)."""
    c = field.centers.detach().double()
    r = field.radii.detach().double()
    axes = [torch.linspace(lo, hi, n, dtype=torch.float64, device=c.device) if n > 1 else
            torch.tensor([lo], dtype=torch.float64, device=c.device) for lo, hi, n in zip(field.lo, field.hi, shape)]
    P = torch.stack(torch.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    g = gsdf.reshape(-1).double()
    nz = g != 0
    P, g = P[nz], g[nz]
    off = P[:, None, :] - c[None]
    dist = off.norm(dim=-1)
    k = (dist - r[None]).argmin(1)
    o = off[torch.arange(len(k)), k]
    dk = dist[torch.arange(len(k)), k]
    gc = torch.zeros_like(c).index_add_(0, k, -g[:, None] * o / dk[:, None])
    gr = torch.zeros_like(r).index_add_(0, k, -g)
    return gc, gr


@pytest.mark.parametrize("method,rq", [("mc", False), ("dmc", True), ("dmc", False)])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("with_deform", [False, True])
def test_field_gradients_match_the_dense_path(cuda_device, method, rq, dtype, with_deform):
    """The fused field backward against the dense path on the field's grid
    (field.materialize, the same values bit for bit): dL/ddeform equal bit for bit,
    dL/d(centres, radii) equal to the dense dL/dsdf carried to the spheres by the
    chain rule in float64 (within 1e-10 relative in float64, 1e-6 in float32)."""
    from diso_gb300 import DiffDMC, DiffMC

    dt = DT[dtype]
    shape = (48, 40, 56)
    c, r, field = _grad_field(cuda_device, dt)
    rng = np.random.default_rng(9)
    dfm = (torch.tensor(rng.uniform(-0.3, 0.3, shape + (3,)), device=cuda_device, dtype=dt).requires_grad_(True)
           if with_deform else None)
    mod = DiffMC(dt) if method == "mc" else DiffDMC(dt)
    kw = {} if method == "mc" else {"return_quads": rq}
    v, f = mod.forward_field(field, shape, deform=dfm, **kw)
    w = torch.randn(v.shape, dtype=dt, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(1))
    (v * w).sum().backward()
    # the dense path on the same values
    s = field.materialize(shape, dt).requires_grad_(True)
    d2 = dfm.detach().clone().requires_grad_(True) if with_deform else None
    v2, f2 = (DiffMC(dt) if method == "mc" else DiffDMC(dt))(s, d2, **kw)
    assert torch.equal(v.detach(), v2.detach()) and torch.equal(f, f2)
    (v2 * w).sum().backward()
    if with_deform:
        assert torch.equal(dfm.grad, d2.grad)
    gc, gr = _chain_rule(field, shape, s.grad)
    scale = max(float(gc.abs().max()), float(gr.abs().max()))
    # float32: the offsets from the centres are taken in float32, as the field's values
    # are, and the gradients are returned in float32
    rtol = 1e-10 if dtype == "float64" else 1e-6
    assert float((c.grad.double() - gc).abs().max()) <= rtol * scale
    assert float((r.grad.double() - gr).abs().max()) <= rtol * scale


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_field_gradients_by_central_differences(cuda_device, method):
    """float64: dL/d(centres, radii) against central differences of the extraction
    itself (h = 1e-6; DMC with exact_grad, the true derivative)."""
    from diso_gb300 import DiffDMC, DiffMC, SphereUnion

    dt = torch.float64
    shape = (40, 36, 44)
    c, r, field = _grad_field(cuda_device, dt, K=3, seed=5)
    mod = DiffMC(dt) if method == "mc" else DiffDMC(dt, exact_grad=True)
    kw = {} if method == "mc" else {"return_quads": True}
    v, _ = mod.forward_field(field, shape, **kw)
    w = torch.randn(v.shape, dtype=dt, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(2))
    (v * w).sum().backward()

    def loss(cc, rr):
        with torch.no_grad():
            vv, _ = mod.forward_field(SphereUnion(cc, rr), shape, **kw)
        assert vv.shape == v.shape  # no change of topology for the small step
        return float((vv * w).sum())

    h = 1e-6
    for k in range(3):
        for a in range(4):
            cp, cm, rp, rm = c.detach().clone(), c.detach().clone(), r.detach().clone(), r.detach().clone()
            if a < 3:
                cp[k, a] += h
                cm[k, a] -= h
                g = float(c.grad[k, a])
            else:
                rp[k] += h
                rm[k] -= h
                g = float(r.grad[k])
            fd = (loss(cp, rp) - loss(cm, rm)) / (2 * h)
            assert abs(fd - g) <= 1e-6 * max(1.0, abs(g)), (k, a, fd, g)
