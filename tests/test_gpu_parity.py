"""Parity of the CUDA path (through the public DiffMC / DiffDMC API and the C ABI)
with the reference's own outputs (golden fixtures) and with the CPU oracle."""
import zlib

import numpy as np
import pytest
import torch

from helpers import (assert_faces_equal, assert_grads_close, assert_verts_close, fixture_names, load_fixture,
                     oracle_grad_rtol)
from oracle import oracle as O

pytestmark = pytest.mark.gpu

DT = {"float32": torch.float32, "float64": torch.float64}


def run(case, sdf_np, def_np, weights=None, exact_grad=False, device="cuda:0", recompute=False):
    from diso_gb300 import DiffDMC, DiffMC

    dt = DT[case["dtype"]]
    sdf = torch.tensor(sdf_np, device=device, requires_grad=True)
    deform = torch.tensor(def_np, device=device, requires_grad=True) if def_np is not None else None
    if case["method"] == "mc":
        verts, faces = DiffMC(dt, recompute=recompute)(sdf, deform, isovalue=case["iso"],
                                                        normalize=case["normalize"])
    else:
        verts, faces = DiffDMC(dt, exact_grad=exact_grad, recompute=recompute)(
            sdf, deform, isovalue=case["iso"], return_quads=case["return_quads"], normalize=case["normalize"])
    out = dict(verts=verts.detach().cpu().numpy(), faces=faces.cpu().numpy(), faces_dtype=str(faces.dtype))
    if weights is not None and verts.shape[0]:
        (verts * torch.tensor(weights, device=device)).sum().backward()
        out["grad_sdf"] = sdf.grad.cpu().numpy()
        if deform is not None:
            out["grad_deform"] = deform.grad.cpu().numpy()
    return out


@pytest.mark.parametrize("recompute", [False, True])
@pytest.mark.parametrize("name", fixture_names())
def test_matches_reference_fixture(cuda_device, name, recompute):
    fx = load_fixture(name)
    c = fx["case"]
    out = run(c, fx["sdf"], fx["deform"], fx.get("weights"), recompute=recompute)
    assert out["faces_dtype"] == fx["faces_dtype"]
    assert_verts_close(out["verts"], fx["verts"], c)
    assert_faces_equal(out["faces"], fx["faces"], c, fx["verts"])
    if "grad_sdf" in fx:
        assert_grads_close(out["grad_sdf"], fx["grad_sdf"], c["dtype"], "grad_sdf")
        if fx["deform"] is not None:
            assert_grads_close(out["grad_deform"], fx["grad_deform"], c["dtype"], "grad_deform")


def _field(kind, shape, rng):
    if kind == "uniform":
        return rng.uniform(-1, 1, shape)
    axes = [np.linspace(-1, 1, n) for n in shape]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    if kind == "sphere":
        return np.sqrt(X * X + Y * Y + Z * Z) - 0.5 + 0.02 * rng.standard_normal(shape)
    if kind == "spheres":
        s = np.full(shape, np.inf)
        for _ in range(6):
            c = rng.uniform(-0.7, 0.7, 3)
            s = np.minimum(s, np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - rng.uniform(0.1, 0.3))
        return s + 0.01 * rng.standard_normal(shape)
    raise ValueError(kind)


ORACLE_CASES = [
    # (method, dtype, field, shape, deform, iso, normalize, return_quads)
    ("mc", "float32", "uniform", (48, 48, 48), 0.45, 0.0, True, False),
    ("dmc", "float32", "uniform", (48, 48, 48), 0.45, 0.0, True, True),
    ("dmc", "float32", "uniform", (33, 40, 35), 0.45, 0.1, True, False),
    ("mc", "float64", "spheres", (37, 20, 65), 0.3, 0.0, True, False),
    ("dmc", "float64", "spheres", (37, 20, 65), 0.3, 0.0, False, True),
    ("dmc", "float64", "uniform", (70, 9, 33), None, -0.2, True, False),
    ("mc", "float32", "sphere", (1, 1, 1), None, 0.0, True, False),
    ("mc", "float32", "uniform", (1, 5, 3), None, 0.0, False, False),
    ("dmc", "float32", "uniform", (2, 1, 64), 0.45, 0.0, True, True),
    ("mc", "float32", "spheres", (128, 128, 128), 0.45, 0.0, True, False),
    ("dmc", "float32", "spheres", (128, 128, 128), 0.45, 0.0, True, True),
    # 64 x 128 rows of one and of two 32-cell segments: 8192 and 16384 segments, whole
    # tiles of the segment scan
    ("mc", "float32", "uniform", (63, 127, 31), None, 0.0, True, False),
    ("dmc", "float32", "spheres", (63, 127, 63), 0.3, 0.0, True, True),
]


@pytest.mark.parametrize("recompute", [False, True])
@pytest.mark.parametrize("method,dtype,field,shape,deform,iso,normalize,rq", ORACLE_CASES)
def test_matches_oracle(cuda_device, method, dtype, field, shape, deform, iso, normalize, rq, recompute):
    rng = np.random.default_rng(zlib.crc32(repr((method, dtype, field, shape)).encode()))
    sdf = _field(field, shape, rng).astype(dtype)
    dfm = rng.uniform(-deform, deform, shape + (3,)).astype(dtype) if deform else None
    case = dict(method=method, dtype=dtype, iso=iso, normalize=normalize, return_quads=rq, shape=shape)
    m = O.MC if method == "mc" else O.DMC
    v_ref, f_ref, info = O.extract(m, sdf, dfm, iso, normalize, rq, dtype)
    w = rng.standard_normal(v_ref.shape).astype(dtype)
    out = run(case, sdf, dfm, w, recompute=recompute)
    if info["empty_guard"]:
        assert out["verts"].shape == (0, 3) and out["faces_dtype"] == "torch.int32"
        return
    assert_verts_close(out["verts"], v_ref, case)
    assert_faces_equal(out["faces"], f_ref, case, v_ref)
    gs, gd = O.backward(m, sdf, dfm, w, iso, normalize, dtype)
    rtol = oracle_grad_rtol(dtype, shape)
    assert_grads_close(out["grad_sdf"], gs, dtype, "grad_sdf", rtol)
    if dfm is not None:
        assert_grads_close(out["grad_deform"], gd, dtype, "grad_deform", rtol)


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_dmc_exact_gradient_matches_oracle(cuda_device, dtype):
    rng = np.random.default_rng(4)
    shape = (20, 21, 22)
    sdf = rng.uniform(-1, 1, shape).astype(dtype)
    dfm = rng.uniform(-0.4, 0.4, shape + (3,)).astype(dtype)
    case = dict(method="dmc", dtype=dtype, iso=0.0, normalize=True, return_quads=True, shape=shape)
    v_ref, _, _ = O.extract(O.DMC, sdf, dfm, 0.0, True, True, dtype)
    w = rng.standard_normal(v_ref.shape).astype(dtype)
    out = run(case, sdf, dfm, w, exact_grad=True)
    gs, gd = O.backward(O.DMC, sdf, dfm, w, 0.0, True, dtype, exact=True)
    rtol = oracle_grad_rtol(dtype, shape)
    assert_grads_close(out["grad_sdf"], gs, dtype, "grad_sdf", rtol)
    assert_grads_close(out["grad_deform"], gd, dtype, "grad_deform", rtol)


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_finite_differences_fp64(cuda_device, method):
    """Central differences (h = 1e-6, float64) on 8 random SDF entries next to
    crossings of a 32^3 grid, and on deform entries."""
    from diso_gb300 import DiffDMC, DiffMC

    rng = np.random.default_rng(8)
    n = 32
    base = torch.tensor(_field("spheres", (n, n, n), rng), device=cuda_device)
    dfm = torch.tensor(rng.uniform(-0.3, 0.3, (n, n, n, 3)), device=cuda_device)
    ext = DiffMC(torch.float64) if method == "mc" else DiffDMC(torch.float64, exact_grad=True)

    def loss(s, d, w):
        v = ext(s, d, return_quads=True)[0] if method == "dmc" else ext(s, d)[0]
        return (v * w).sum()

    s = base.clone().requires_grad_(True)
    d = dfm.clone().requires_grad_(True)
    v = ext(s, d)[0]
    w = torch.tensor(rng.standard_normal(tuple(v.shape)), device=cuda_device)
    loss(s, d, w).backward()
    gs, gd = s.grad, d.grad
    h = 1e-6
    cand = torch.nonzero(gs.abs() > 1e-3).cpu().numpy()
    for i in cand[rng.choice(len(cand), 8, replace=False)]:
        i = tuple(int(k) for k in i)
        sp, sm = base.clone(), base.clone()
        sp[i] += h
        sm[i] -= h
        with torch.no_grad():
            fd = (loss(sp, dfm, w) - loss(sm, dfm, w)).item() / (2 * h)
        assert abs(fd - gs[i].item()) <= 1e-5 * max(1.0, abs(fd)), (i, fd, gs[i].item())
    cand = torch.nonzero(gd.abs() > 1e-3).cpu().numpy()
    for j in cand[rng.choice(len(cand), 4, replace=False)]:
        j = tuple(int(k) for k in j)
        dp, dm = dfm.clone(), dfm.clone()
        dp[j] += h
        dm[j] -= h
        with torch.no_grad():
            fd = (loss(base, dp, w) - loss(base, dm, w)).item() / (2 * h)
        assert abs(fd - gd[j].item()) <= 1e-6 * max(1.0, abs(fd)), (j, fd, gd[j].item())


def test_noncontiguous_inputs_and_side_stream(cuda_device):
    from diso_gb300 import DiffMC

    rng = np.random.default_rng(1)
    base = torch.tensor(_field("spheres", (24, 30, 26), rng).astype(np.float32), device=cuda_device)
    t = base.permute(2, 0, 1)  # non-contiguous view [26, 24, 30]
    ref_v, ref_f, _ = O.extract(O.MC, t.contiguous().cpu().numpy(), None, 0.0, True, False, "float32")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        v, f = DiffMC(torch.float32)(t)
    s.synchronize()
    assert np.array_equal(f.cpu().numpy(), ref_f)
    assert np.abs(v.cpu().numpy() - ref_v).max() < 1e-6


def test_backward_is_deterministic(cuda_device):
    from diso_gb300 import DiffDMC

    rng = np.random.default_rng(2)
    sdf = torch.tensor(rng.uniform(-1, 1, (40, 40, 40)).astype(np.float32), device=cuda_device)
    grads = []
    for _ in range(2):
        s = sdf.clone().requires_grad_(True)
        v, _ = DiffDMC(torch.float32)(s, return_quads=True)
        (v * v).sum().backward()
        grads.append(s.grad.clone())
    assert torch.equal(grads[0], grads[1])


def test_second_backward_and_forward_without_backward(cuda_device):
    # the gradient buffers are zeroed during the forward and filled by the first
    # backward; a second backward of the same graph (retain_graph) and forwards whose
    # outputs are dropped before any backward give the same gradients
    from diso_gb300 import DiffDMC, DiffMC

    rng = np.random.default_rng(3)
    sdf = torch.tensor(rng.uniform(-1, 1, (36, 28, 44)).astype(np.float32), device=cuda_device)
    dfm = torch.tensor(rng.uniform(-0.3, 0.3, (36, 28, 44, 3)).astype(np.float32), device=cuda_device)
    for mod in (DiffMC(torch.float32), DiffDMC(torch.float32)):
        s = sdf.clone().requires_grad_(True)
        d = dfm.clone().requires_grad_(True)
        for _ in range(3):  # forwards without backward: their zeroed buffers are released
            mod(s, d)
        v, _ = mod(s, d)
        loss = (v * v).sum()
        loss.backward(retain_graph=True)
        g1, d1 = s.grad.clone(), d.grad.clone()
        loss.backward()
        assert torch.equal(s.grad, 2 * g1) and torch.equal(d.grad, 2 * d1)
        assert g1.abs().sum() > 0 and d1.abs().sum() > 0


@pytest.mark.parametrize("nz", [36, 35])
def test_gradient_zeroing_paths(cuda_device, nz):
    # buffers given to diso_zero_grads are zero once the next forward on the same
    # stream has run: written by its count and emit (rows of 36 floats: the TMA count;
    # bytes past the last 16-byte vector included), by memsets when the count finds no
    # surface, on the side stream otherwise (rows of 35 floats, a misaligned buffer, a
    # count on another stream)
    from diso_gb300 import _native as N

    ex = N.Extractor(N.DMC, torch.float32)
    rng = np.random.default_rng(5)
    g = torch.tensor(rng.uniform(-1, 1, (21, 18, nz)).astype(np.float32), device=cuda_device)
    iso, pad = N.iso_values(0.0, torch.float32)
    seg = torch.empty(N.Extractor.segment_slots(g.shape), dtype=torch.int64, device=cuda_device)

    def forward(grid):
        c = ex.count(grid, iso, pad, seg)
        if not c.empty:
            verts = torch.empty((c.n_verts, 3), device=cuda_device)
            quads = torch.empty((c.n_faces, 4), dtype=torch.int64, device=cuda_device)
            ex.emit(grid, None, iso, pad, seg, True, verts, quads)
        return c

    def nans(n, offset=0):
        return torch.full((n + offset,), float("nan"), device=cuda_device)[offset:]

    def zeroed(*ts):
        torch.cuda.synchronize()
        return all(bool(torch.all(t == 0)) for t in ts if t is not None)

    a, b = nans(g.numel() + 2), nans(3 * g.numel() + 1)
    ex.zero_grads(a, b)
    assert not forward(g).empty
    assert zeroed(a, b)
    a = nans(1000)
    ex.zero_grads(a, None)
    forward(g)
    assert zeroed(a)
    a, b = nans(g.numel()), nans(3 * g.numel())
    ex.zero_grads(a, b)
    assert forward(g + 2).empty
    assert zeroed(a, b)
    a, b = nans(999, offset=1), nans(77)
    assert a.data_ptr() % 16 != 0
    ex.zero_grads(a, b)
    forward(g)
    assert zeroed(a, b)
    a1, a2 = nans(5000), nans(7000)
    ex.zero_grads(a1, None)
    ex.zero_grads(a2, None)  # replaces the first call's buffers
    forward(g)
    assert zeroed(a2)
    a, b = nans(3000), nans(50)
    ex.zero_grads(a, b)
    other = torch.cuda.Stream(cuda_device)
    other.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(other):
        c = forward(g)
    assert zeroed(a, b) and c.n_faces > 0


@pytest.mark.parametrize("method", ["mc", "dmc"])
def test_single_call_forward_and_capacity_fallback(cuda_device, method):
    # a module that has seen a grid of this shape runs the forward as one native call
    # into outputs sized from that grid; a larger surface than that falls back to an
    # emit of the exact sizes; results equal those of a fresh module either way
    from diso_gb300 import DiffDMC, DiffMC

    mk = (lambda: DiffMC(torch.float32)) if method == "mc" else (lambda: DiffDMC(torch.float32))
    rng = np.random.default_rng(4)
    shape = (40, 33, 47)
    small = torch.tensor(_field("spheres", shape, rng).astype(np.float32), device=cuda_device)
    big = torch.tensor(rng.uniform(-1, 1, shape).astype(np.float32), device=cuda_device)
    w = torch.tensor(rng.uniform(-1, 1, (200000, 3)).astype(np.float32), device=cuda_device)

    def run(mod, grid):
        s = grid.clone().requires_grad_(True)
        v, f = mod(s)
        (v * w[: v.shape[0]]).sum().backward()
        return v.detach().clone(), f.clone(), s.grad.clone()

    warm = mk()
    for grid in (small, big, big, small):  # fallback, then fits, then fits with room
        got = run(warm, grid)
        ref = run(mk(), grid)
        for a, b in zip(got, ref):
            assert a.shape == b.shape and torch.equal(a, b)


def test_empty_guard_and_errors(cuda_device):
    from diso_gb300 import DiffDMC, DiffMC

    g = torch.ones(5, 6, 7, device=cuda_device)
    v, f = DiffMC(torch.float32)(g)
    assert v.shape == (0, 3) and f.shape == (0, 3) and f.dtype == torch.int32
    v, f = DiffDMC(torch.float32)(g - 2, return_quads=False)
    assert v.shape == (0, 3) and f.shape == (0, 4) and f.dtype == torch.int32
    with pytest.raises(RuntimeError):
        DiffMC(torch.float64)(g)
    with pytest.raises(RuntimeError):
        DiffMC(torch.float32)(g.cpu())
