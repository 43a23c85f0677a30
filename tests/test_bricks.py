"""Narrow-band input on the CPU: the band's layout and its dense grid (BrickGrid), the
claim that a band cut from a dense grid keeps the dense grid's meshes (checked with the
float64 oracle on both grids), and the C entry points' argument checks (no GPU call)."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import oracle as O


def _sphere(n, r=0.5, dtype=torch.float64):
    a = torch.linspace(-1, 1, n, dtype=dtype)
    X, Y, Z = torch.meshgrid(a, a, a, indexing="ij")
    return torch.sqrt(X * X + Y * Y + Z * Z) - r


def test_brick_layout_and_dense_round_trip():
    from diso_gb300.bricks import BrickGrid

    g = torch.Generator().manual_seed(0)
    sdf = torch.randn((19, 21, 17), generator=g, dtype=torch.float64)
    dfm = torch.rand((19, 21, 17, 3), generator=g, dtype=torch.float64)
    band = BrickGrid.from_dense(sdf, 0.1, deform=dfm)
    assert tuple(band.index.shape) == (3, 3, 3) and band.index.dtype == torch.int32
    # a random field crosses everywhere: every brick present, slots in x-major order
    assert torch.equal(band.index.flatten(), torch.arange(27, dtype=torch.int32))
    # slot (bx, by, bz), point (i, j, k) holds sdf[8 bx + i, 8 by + j, 8 bz + k]
    bx, by, bz = 1, 2, 0
    s = band.index[bx, by, bz]
    assert torch.equal(band.values[s, :3, :5, :8], sdf[8:11, 16:21, 0:8])
    assert torch.equal(band.deform[s, :3, :5, :8], dfm[8:11, 16:21, 0:8])
    d, dd = band.dense()
    assert torch.equal(d, sdf) and torch.equal(dd, dfm)


@pytest.mark.parametrize("iso", [0.0, 0.2, -0.1])
def test_band_of_a_sphere_keeps_every_side(iso):
    from diso_gb300.bricks import BrickGrid
    from diso_gb300._native import BRICK_INSIDE, BRICK_OUTSIDE

    sdf = _sphere(61, 0.6)
    band = BrickGrid.from_dense(sdf, iso, band=0.02)
    d, _ = band.dense()
    assert torch.equal(d >= iso, sdf >= iso)
    idx = band.index
    assert (idx == BRICK_OUTSIDE).any() and (idx == BRICK_INSIDE).any() and 0 < band.count < idx.numel()
    # the present bricks hold the original values; absent ones +-background
    present = (d == sdf)
    assert present.sum() >= band.count * 8 ** 3 * 0.5
    assert set(torch.unique(d[~present]).tolist()) <= {band.background, -band.background}


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_band_meshes_equal_dense_meshes_by_the_oracle(method):
    # the oracle on the band's dense grid and on the original grid: the same mesh, so a
    # band cut by from_dense loses nothing near the surface
    from diso_gb300.bricks import BrickGrid

    n = 37
    sdf = _sphere(n, 0.55) + 0.05 * torch.sin(7 * torch.linspace(0, 1, n, dtype=torch.float64))[None, None, :]
    g = torch.Generator().manual_seed(3)
    dfm = (torch.rand((n, n, n, 3), generator=g, dtype=torch.float64) - 0.5) * 0.6
    band = BrickGrid.from_dense(sdf, 0.0, deform=dfm)
    d, dd = band.dense()
    m = O.MC if method == "mc" else O.DMC
    v0, f0, _ = O.extract(m, sdf.numpy(), dfm.numpy(), 0.0, True, True, "float64")
    v1, f1, _ = O.extract(m, d.numpy(), dd.numpy(), 0.0, True, True, "float64")
    assert np.array_equal(f0, f1) and np.array_equal(v0, v1)
    w = np.random.default_rng(1).standard_normal(v0.shape)
    gs0, gd0 = O.backward(m, sdf.numpy(), dfm.numpy(), w, 0.0, True, "float64")
    gs1, gd1 = O.backward(m, d.numpy(), dd.numpy(), w, 0.0, True, "float64")
    # the oracle's OpenMP sums are not in a fixed order: equal up to their rounding
    for g0, g1 in ((gs0, gs1), (gd0, gd1)):
        assert np.abs(g0 - g1).max() <= 1e-12 * np.abs(g0).max()
    # no gradient outside the bricks
    out = (d != sdf).numpy()
    assert not gs0[out].any()


def test_brick_grid_rejects_bad_shapes():
    from diso_gb300.bricks import BrickGrid

    idx = torch.zeros((2, 2, 2), dtype=torch.int32)
    vals = torch.zeros((1, 8, 8, 8))
    with pytest.raises(RuntimeError, match="int32 of shape"):
        BrickGrid((16, 16, 17), idx, vals)
    with pytest.raises(RuntimeError, match="int32 of shape"):
        BrickGrid((16, 16, 16), idx.long(), vals)
    with pytest.raises(RuntimeError, match=r"\[K, 8, 8, 8\]"):
        BrickGrid((16, 16, 16), idx, torch.zeros((1, 8, 8, 4)))
    with pytest.raises(RuntimeError, match="deform"):
        BrickGrid((16, 16, 16), idx, vals, deform=torch.zeros((1, 8, 8, 8, 2)))
    with pytest.raises(RuntimeError, match="background"):
        BrickGrid((16, 16, 16), idx, vals, background=0.0)


@pytest.fixture(scope="module")
def lib():
    from diso_gb300.build import build

    build()
    from diso_gb300 import _native

    return _native.lib()


def test_brick_entry_points_check_their_arguments(lib):
    from diso_gb300 import _native as N

    h = ctypes.c_void_p()
    assert lib.diso_create(1, 0, ctypes.byref(h)) == 0
    c = N.Counts()
    d = N.BrickGridDesc()
    p = ctypes.c_void_p(4096)
    d.dims[:] = (16, 16, 16)
    d.index = None
    d.count = 1
    d.values = 4096
    d.background = 1.0
    fwd = lambda: lib.diso_forward_bricks(h, ctypes.byref(d), 0.0, 1.0, p, 1, p, 16, p, 16, None, ctypes.byref(c))
    assert fwd() == 1 and b"null brick grid or index" in lib.diso_last_error()
    d.index = 4096
    d.background = 0.0
    assert fwd() == 1 and b"background" in lib.diso_last_error()
    d.background = float("nan")
    assert fwd() == 1 and b"background" in lib.diso_last_error()
    d.background = 1.0
    d.dims[:] = (16, 0, 16)
    assert fwd() == 1 and b"grid dims" in lib.diso_last_error()
    d.dims[:] = (16, 16, 16)
    d.count = -1
    assert fwd() == 1 and b"negative brick count" in lib.diso_last_error()
    d.count = 1
    d.values = None
    assert fwd() == 1 and b"null brick values" in lib.diso_last_error()
    d.values = 4096
    assert lib.diso_forward_bricks(h, ctypes.byref(d), 0.0, 1.0, None, 1, p, 16, p, 16, None, ctypes.byref(c)) == 1
    bwd = lambda gv, gval, gdef: lib.diso_backward_bricks(h, ctypes.byref(d), 0.0, 1.0, p, 1, 0, gv, gval, gdef, None)
    assert bwd(None, p, None) == 1 and b"grad_verts" in lib.diso_last_error()
    assert bwd(p, None, None) == 1 and b"grad_values" in lib.diso_last_error()
    d.deform = 4096
    assert bwd(p, p, None) == 1 and b"needs grad_deform" in lib.diso_last_error()
    assert lib.diso_bricks_materialize(5, ctypes.byref(d), p, None, None) == 1
    d.deform = None
    assert lib.diso_bricks_materialize(0, ctypes.byref(d), p, p, None) == 1
    assert b"without one" in lib.diso_last_error()
    # the dense path's index limits (counts of larger grids are checked after the count)
    assert lib.diso_forward_count(h, p, 16385, 16, 16, 0.0, 1.0, p, None, ctypes.byref(c)) == 1
    assert b"too large" in lib.diso_last_error()
    assert lib.diso_forward_count(h, p, 8192, 8192, 2048, 0.0, 1.0, p, None, ctypes.byref(c)) == 1
    assert b"too large" in lib.diso_last_error()
    lib.diso_destroy(h)
