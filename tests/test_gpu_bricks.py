"""Narrow-band extraction (DiffMC / DiffDMC.forward_bricks over diso_forward_bricks /
diso_backward_bricks) against the dense path on the band's dense grid (BrickGrid.dense),
which the other parity tests tie to the reference, and against the float64 oracle:
vertices and faces identical bit for bit, gradients equal to the dense gradients at the
bricks' points.  Then a 1024^3 band, past the dense path's 32-bit limit, against the dense
extraction of the sub-grid that holds its surface."""
import numpy as np
import pytest
import torch

from helpers import assert_faces_equal, assert_grads_close, assert_verts_close

pytestmark = pytest.mark.gpu

DT = {"float32": torch.float32, "float64": torch.float64}


def _grid(kind, shape, dtype, device):
    g = torch.Generator().manual_seed(11)
    axes = [torch.linspace(-1, 1, n, dtype=torch.float64) for n in shape]
    X, Y, Z = torch.meshgrid(*axes, indexing="ij")
    if kind == "sphere":
        s = torch.sqrt(X * X + Y * Y + Z * Z) - 0.6
    elif kind == "cube":  # the round cube of the reference's README
        q = torch.stack([torch.clamp(c.abs() - 0.5, min=0) for c in (X, Y, Z)], -1)
        s = q.norm(dim=-1) - 0.1
    elif kind == "waves":  # a surface through the grid's faces
        s = Z - 0.3 * torch.sin(3 * X) * torch.cos(2 * Y)
    else:  # dense random: every brick present
        s = torch.rand(shape, generator=g, dtype=torch.float64) * 2 - 1
    d = (torch.rand(tuple(shape) + (3,), generator=g, dtype=torch.float64) - 0.5) * 0.9
    return s.to(dtype).to(device), d.to(dtype).to(device)


CASES = [
    # (kind, shape, iso, normalize, band)
    ("sphere", (64, 64, 64), 0.0, True, 0.0),
    ("cube", (45, 37, 53), 0.0, True, 0.05),
    ("waves", (40, 33, 29), 0.1, False, 0.0),
    ("random", (27, 19, 24), 0.2, True, 0.0),
]


@pytest.mark.parametrize("method,rq", [("mc", False), ("dmc", True), ("dmc", False)])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("deform", [False, True])
@pytest.mark.parametrize("kind,shape,iso,normalize,band", CASES)
def test_band_matches_dense(cuda_device, method, rq, dtype, deform, kind, shape, iso, normalize, band):
    from diso_gb300 import BrickGrid, DiffDMC, DiffMC

    dt = DT[dtype]
    sdf, dfm = _grid(kind, shape, dt, cuda_device)
    bg = BrickGrid.from_dense(sdf, iso, band=band, deform=dfm if deform else None)
    dense, ddense = bg.dense()
    # the library's materialization is the same grid
    ms, md = bg.materialize()
    assert torch.equal(ms, dense) and (md is None or torch.equal(md, ddense))
    bg.values.requires_grad_(True)
    if deform:
        bg.deform.requires_grad_(True)
    mod = DiffMC(dt) if method == "mc" else DiffDMC(dt)
    if method == "mc":
        v, f = mod.forward_bricks(bg, isovalue=iso, normalize=normalize)
    else:
        v, f = mod.forward_bricks(bg, isovalue=iso, return_quads=rq, normalize=normalize)
    ds = dense.clone().requires_grad_(True)
    dd = ddense.clone().requires_grad_(True) if deform else None
    if method == "mc":
        v_ref, f_ref = mod(ds, dd, isovalue=iso, normalize=normalize)
    else:
        v_ref, f_ref = mod(ds, dd, isovalue=iso, return_quads=rq, normalize=normalize)
    assert v.shape[0] > 0
    assert torch.equal(v, v_ref), "vertices differ from the dense path"
    assert torch.equal(f, f_ref), "faces differ from the dense path"
    w = torch.randn(v.shape, dtype=dt, device=cuda_device, generator=torch.Generator(cuda_device).manual_seed(5))
    (v * w).sum().backward()
    (v_ref * w).sum().backward()
    # the dense gradients at the bricks' points, and none elsewhere
    idx = bg.index.reshape(-1).long()
    slot_of = torch.full((bg.count,), -1, dtype=torch.long, device=cuda_device)
    slot_of[idx[idx >= 0]] = torch.nonzero(idx >= 0).flatten()
    from diso_gb300.bricks import _to_bricks, brick_dims

    nb = brick_dims(shape)
    gb = _to_bricks(ds.grad, nb, 0.0)[slot_of]
    assert torch.equal(bg.values.grad, gb), "dL/dvalues differs from the dense gradient"
    assert not _to_bricks(ds.grad, nb, 0.0)[idx < 0].any(), "dense gradient outside the bricks"
    if deform:
        gdb = _to_bricks(dd.grad, nb, 0.0)[slot_of]
        assert torch.equal(bg.deform.grad, gdb), "dL/ddeform differs from the dense gradient"


@pytest.mark.parametrize("method", ["mc", "dmc"])
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_band_against_the_oracle(cuda_device, method, dtype):
    from diso_gb300 import BrickGrid, DiffDMC, DiffMC
    from oracle import oracle as O

    dt = DT[dtype]
    sdf, dfm = _grid("sphere", (48, 40, 56), dt, cuda_device)
    bg = BrickGrid.from_dense(sdf, 0.0, band=0.03, deform=dfm)
    bg.values.requires_grad_(True)
    bg.deform.requires_grad_(True)
    mod = DiffMC(dt) if method == "mc" else DiffDMC(dt)
    v, f = mod.forward_bricks(bg) if method == "mc" else mod.forward_bricks(bg, return_quads=True)
    dense, ddense = bg.dense()
    s_np, d_np = dense.cpu().numpy(), ddense.cpu().numpy()
    m = O.MC if method == "mc" else O.DMC
    v_ref, f_ref, _ = O.extract(m, s_np, d_np, 0.0, True, True, dtype)
    case = dict(method=method, dtype=dtype, iso=0.0, normalize=True, return_quads=True, shape=tuple(dense.shape))
    assert_verts_close(v.detach().cpu().numpy(), v_ref, case)
    assert_faces_equal(f.cpu().numpy(), f_ref, case)
    w = np.random.default_rng(2).standard_normal(v_ref.shape).astype(dtype)
    (v * torch.tensor(w, device=cuda_device)).sum().backward()
    gs_ref, gd_ref = O.backward(m, s_np, d_np, w, 0.0, True, dtype)
    from diso_gb300.bricks import _to_bricks, brick_dims

    nb = brick_dims(dense.shape)
    idx = bg.index.reshape(-1).long().cpu()
    sel = torch.nonzero(idx >= 0).flatten()
    gs_b = _to_bricks(torch.tensor(gs_ref), nb, 0.0)[sel].numpy()
    gd_b = _to_bricks(torch.tensor(gd_ref), nb, 0.0)[sel].numpy()
    assert_grads_close(bg.values.grad.cpu().numpy(), gs_b, dtype, "grad_values")
    assert_grads_close(bg.deform.grad.cpu().numpy(), gd_b, dtype, "grad_deform")


def test_band_index_errors(cuda_device):
    from diso_gb300 import BrickGrid, DiffDMC

    sdf, _ = _grid("sphere", (32, 32, 32), torch.float32, cuda_device)
    bg = BrickGrid.from_dense(sdf, 0.0)
    mod = DiffDMC(torch.float32)
    bad = bg.index.clone()
    bad[bad >= 0] = bad[bad >= 0].max() + 1  # a slot past the values
    with pytest.raises(RuntimeError, match="neither a slot"):
        mod.forward_bricks(BrickGrid(bg.dims, bad, bg.values, background=bg.background))
    bad = bg.index.clone()
    bad[bad == -1] = -7  # an unknown tag
    with pytest.raises(RuntimeError, match="neither a slot"):
        mod.forward_bricks(BrickGrid(bg.dims, bad, bg.values, background=bg.background))
    twice = bg.index.clone()
    pres = torch.nonzero(twice.reshape(-1) >= 0).flatten()
    twice.reshape(-1)[pres[1]] = twice.reshape(-1)[pres[0]]
    with pytest.raises(RuntimeError, match="two bricks"):
        mod.forward_bricks(BrickGrid(bg.dims, twice, bg.values, background=bg.background))
    # the extractor still works afterwards
    v, f = mod.forward_bricks(bg)
    v2, f2 = mod(bg.dense()[0])
    assert torch.equal(v, v2) and torch.equal(f, f2)


def test_band_without_surface_and_empty(cuda_device):
    from diso_gb300 import BrickGrid, DiffMC

    dims = (40, 24, 33)
    nb = tuple((n + 7) // 8 for n in dims)
    idx = torch.full(nb, -1, dtype=torch.int32, device=cuda_device)
    vals = torch.zeros((0, 8, 8, 8), device=cuda_device)
    v, f = DiffMC(torch.float32).forward_bricks(BrickGrid(dims, idx, vals))
    assert v.shape == (0, 3) and f.shape == (0, 3)
    # an inside brick at the grid's edge meets the pad: a surface without present bricks
    idx[0, 0, 0] = -2
    bg = BrickGrid(dims, idx, vals)
    v, f = DiffMC(torch.float32).forward_bricks(bg)
    v2, f2 = DiffMC(torch.float32)(bg.dense()[0])
    assert v.shape[0] > 0 and torch.equal(v, v2) and torch.equal(f, f2)


def _sphere_band(dims, centre, radius, box, dtype, device, deform):
    """A band of the sphere |p - centre| - radius (index units, scaled by 1/64) whose
    bricks lie in box = (origin, size) (multiples of 8): bricks whose centre is within
    12 of the surface are present, the others tagged by the side of their centre."""
    from diso_gb300 import BrickGrid

    nb = tuple((n + 7) // 8 for n in dims)
    o, m = box
    b0, bm = o // 8, m // 8
    r = torch.arange(bm, dtype=torch.float64)
    cx, cy, cz = torch.meshgrid(r, r, r, indexing="ij")
    cen = torch.stack([(b0 + c) * 8 + 3.5 for c in (cx, cy, cz)], -1)
    dc = (cen - torch.tensor(centre, dtype=torch.float64)).norm(dim=-1) - radius
    present = dc.abs() <= 12.0
    sub = torch.where(present, 0, torch.where(dc > 0, -1, -2)).to(torch.int32)
    k = int(present.sum())
    sub[present] = torch.arange(k, dtype=torch.int32)
    idx = torch.full(nb, -1, dtype=torch.int32)
    idx[b0:b0 + bm, b0:b0 + bm, b0:b0 + bm] = sub
    pb = torch.nonzero(present)  # [K, 3] brick coordinates in the box, in slot order
    lr = torch.arange(8, dtype=torch.float64)
    lx, ly, lz = torch.meshgrid(lr, lr, lr, indexing="ij")
    pts = torch.stack([(b0 + pb[:, a, None, None, None]) * 8 + l[None] for a, l in enumerate((lx, ly, lz))], -1)
    vals = ((pts - torch.tensor(centre, dtype=torch.float64)).norm(dim=-1) - radius) / 64.0
    g = torch.Generator().manual_seed(4)
    dfm = ((torch.rand(tuple(vals.shape) + (3,), generator=g, dtype=torch.float64) - 0.5) * 0.8 if deform else None)
    band = BrickGrid(dims, idx.to(device), vals.to(dtype).to(device),
                     dfm.to(dtype).to(device) if dfm is not None else None, background=1.0)
    sub_band = BrickGrid((m, m, m), sub.to(device), band.values, band.deform, background=1.0)
    return band, sub_band


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_band_beyond_the_dense_limit(cuda_device, method):
    # 1024^3 points: the dense path refuses it (32-bit counts for the worst case); the
    # band's surface lies in the sub-grid [536, 872)^3, whose dense extraction (normalize
    # off) gives the same mesh shifted by 536 in every coordinate
    from diso_gb300 import DiffDMC, DiffMC

    dims = (1024, 1024, 1024)
    o, m = 536, 336
    band, sub = _sphere_band(dims, (700.3, 690.6, 710.2), 150.0, (o, m), torch.float64, cuda_device, True)
    band.values.requires_grad_(True)
    band.deform.requires_grad_(True)
    mod = DiffMC(torch.float64) if method == "mc" else DiffDMC(torch.float64)
    kw = {} if method == "mc" else {"return_quads": True}
    v, f = mod.forward_bricks(band, normalize=False, **kw)
    ds, dd = sub.dense()
    ds.requires_grad_(True)
    dd.requires_grad_(True)
    v2, f2 = mod(ds, dd, normalize=False, **kw)
    assert v.shape[0] > 100_000
    assert torch.equal(f, f2), "faces differ from the sub-grid's"
    assert (v - (v2 + o)).abs().max().item() < 1e-9, "vertices differ from the sub-grid's"
    w = torch.randn(v.shape, dtype=torch.float64, device=cuda_device,
                    generator=torch.Generator(cuda_device).manual_seed(9))
    (v * w).sum().backward()
    (v2 * w).sum().backward()
    from diso_gb300.bricks import _to_bricks, brick_dims

    nb = brick_dims((m, m, m))
    sel = torch.nonzero(sub.index.reshape(-1) >= 0).flatten()
    gs = _to_bricks(ds.grad, nb, 0.0)[sel]
    gd = _to_bricks(dd.grad, nb, 0.0)[sel]
    assert (band.values.grad - gs).abs().max().item() <= 1e-12 * gs.abs().max().item()
    assert (band.deform.grad - gd).abs().max().item() <= 1e-12 * gd.abs().max().item()
