"""Parity of the mesh consumers on the GPU (diso_gb300.mesh over diso_mesh_*) with
the CPU oracle (oracle/mesh.py): normals, weld, OBJ text and PLY bytes, on the
extractor's own meshes and on constructed ones."""
import math

import numpy as np
import pytest
import torch

from oracle import mesh as M

pytestmark = pytest.mark.gpu


def _spheres(n, rng, dtype):
    ax = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
    s = np.full((n, n, n), np.inf)
    for _ in range(5):
        c = rng.uniform(-0.6, 0.6, 3)
        s = np.minimum(s, np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - rng.uniform(0.15, 0.35))
    return (s + 0.01 * rng.standard_normal(s.shape)).astype(dtype)


def _meshes(device, dtype):
    from diso_gb300 import DiffDMC, DiffMC

    rng = np.random.default_rng(11)
    tdt = torch.float32 if dtype == "float32" else torch.float64
    sdf = torch.tensor(_spheres(40, rng, dtype), device=device)
    dfm = torch.tensor(rng.uniform(-0.3, 0.3, (40, 40, 40, 3)).astype(dtype), device=device)
    out = {"mc": DiffMC(tdt)(sdf, dfm), "dmc_quads": DiffDMC(tdt)(sdf, dfm, return_quads=True),
           "dmc_tris": DiffDMC(tdt)(sdf, dfm)}
    return {k: (v.detach(), f) for k, (v, f) in out.items()}


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_vertex_normals_match_oracle_and_repeat(cuda_device, dtype):
    from diso_gb300 import mesh

    tol = 2e-6 if dtype == "float32" else 1e-9
    for name, (v, f) in _meshes(cuda_device, dtype).items():
        got = mesh.vertex_normals(v, f)
        ref = M.vertex_normals(v.cpu().numpy(), f.cpu().numpy())
        assert got.shape == v.shape and got.dtype == v.dtype
        assert np.abs(got.cpu().numpy() - ref).max() <= tol, name
        assert torch.equal(got, mesh.vertex_normals(v, f)), name


def test_weld_matches_oracle(cuda_device):
    from diso_gb300 import DiffMC, mesh

    # |x| + |y| + |z| - 6 on integer points is exactly zero on an octahedron of grid
    # points, each the end of several crossing edges (t = 1): MC puts a vertex on
    # every one of them, so positions repeat
    n = 24
    ax = np.abs(np.arange(n, dtype=np.float32) - 11)
    sdf = torch.tensor(ax[:, None, None] + ax[None, :, None] + ax[None, None, :] - 6, device=cuda_device)
    v, f = DiffMC(torch.float32)(sdf)
    rng = np.random.default_rng(2)
    vv = rng.integers(0, 6, (3000, 3)).astype(np.float64) / 5 + rng.choice([0, 1e-7], (3000, 1))
    ff = rng.integers(0, 3000, (4000, 4))
    cases = [(v.detach(), f, 0.0), (v.detach(), f, 1e-3), (torch.tensor(vv, device=cuda_device),
                                                           torch.tensor(ff, device=cuda_device), 0.0),
             (torch.tensor(vv, device=cuda_device), torch.tensor(ff, device=cuda_device), 1e-4)]
    for v_, f_, tol in cases:
        gv, gf = mesh.weld(v_, f_, tol)
        rv, rf = M.weld(v_.cpu().numpy(), f_.cpu().numpy(), tol)
        assert np.array_equal(gv.cpu().numpy(), rv) and np.array_equal(gf.cpu().numpy(), rf), tol
    assert M.weld(v.detach().cpu().numpy(), f.cpu().numpy())[0].shape[0] < v.shape[0]  # the case merges


def _special_mesh(dtype):
    vals = [0.0, -0.0, 1 / 512, 3 / 512, -5 / 512, 1e-9, -1e-9, 0.123456785, 2.5e-9, 511.99999999, 1e7 + 0.5,
            123456.78901234567, math.nan, math.inf, -math.inf]
    rng = np.random.default_rng(4)
    v = np.concatenate([np.array(vals * 3).reshape(-1, 3), rng.uniform(-2, 2, (500, 3))]).astype(dtype)
    f = rng.integers(0, v.shape[0], (300, 3))
    return v, f


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_obj_text_matches_oracle(cuda_device, dtype):
    from diso_gb300 import mesh

    v, f = _special_mesh(dtype)
    tv, tf = torch.tensor(v, device=cuda_device), torch.tensor(f, device=cuda_device)
    assert mesh.obj_text(tv, tf).cpu().numpy().tobytes() == M.obj_text(v, f)
    nrm = M.vertex_normals(np.nan_to_num(v, posinf=0, neginf=0), f).astype(dtype)
    got = mesh.obj_text(tv, tf, torch.tensor(nrm, device=cuda_device)).cpu().numpy().tobytes()
    assert got == M.obj_text(v, f, nrm)
    for name, (mv, mf) in _meshes(cuda_device, dtype).items():
        assert mesh.obj_text(mv, mf).cpu().numpy().tobytes() == M.obj_text(mv.cpu().numpy(), mf.cpu().numpy()), name


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_ply_and_files_match_oracle(cuda_device, dtype, tmp_path):
    from diso_gb300 import mesh

    for name, (v, f) in _meshes(cuda_device, dtype).items():
        nrm = mesh.vertex_normals(v, f)
        for normals in (None, nrm):
            ref = M.ply_bytes(v.cpu().numpy(), f.cpu().numpy(), None if normals is None else normals.cpu().numpy())
            path = tmp_path / f"{name}.ply"
            mesh.write_ply(str(path), v, f, normals)
            assert path.read_bytes() == ref, name
        path = tmp_path / f"{name}.obj"
        mesh.write_obj(str(path), v, f, nrm)
        assert path.read_bytes() == M.obj_text(v.cpu().numpy(), f.cpu().numpy(), nrm.cpu().numpy())


def test_face_index_out_of_range_is_an_error(cuda_device):
    from diso_gb300 import mesh

    v = torch.rand(10, 3, device=cuda_device)
    for bad in (10, -1):
        f = torch.tensor([[0, 1, 2], [3, 4, bad]], device=cuda_device)
        with pytest.raises(RuntimeError, match="out of range"):
            mesh.vertex_normals(v, f)
        with pytest.raises(RuntimeError, match="out of range"):
            mesh.weld(v, f)
    ok = mesh.vertex_normals(v, torch.tensor([[0, 1, 2]], device=cuda_device))  # the extractor is still usable
    assert torch.isfinite(ok).all()
