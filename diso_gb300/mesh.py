"""Mesh consumers on the GPU for the meshes DiffMC / DiffDMC return: area-weighted
vertex normals, vertex welding, and OBJ / binary PLY files written from device
memory.

The reference hands its meshes to trimesh on the host and exports them there
(test/example.py:71-73: ``trimesh.Trimesh(vertices, faces, process=False).export``
to OBJ).  Here the text and the binary bodies are produced by CUDA kernels
(``diso_mesh_*`` in include/diso_gb300.h) and only the finished bytes cross to the
host.  Vertices are [V, 3] float32 / float64 CUDA tensors, faces [F, 3] or [F, 4]
integer CUDA tensors (triangles, or DMC quads with ``return_quads=True``).
"""
from __future__ import annotations

import torch

from . import _native as N

_extractors = {}


def _extractor(dtype, device):
    key = (dtype, device)
    ex = _extractors.get(key)
    if ex is None:
        with torch.cuda.device(device):
            ex = _extractors[key] = N.Extractor(N.MC, dtype)
    return ex


def _inputs(verts, faces, normals=None):
    if not verts.is_cuda or not faces.is_cuda or faces.device != verts.device:
        raise RuntimeError("verts and faces must be CUDA tensors on one device")
    if verts.dtype not in (torch.float32, torch.float64):
        raise RuntimeError(f"verts must be float32 or float64, got {verts.dtype}")
    if verts.dim() != 2 or verts.shape[1] != 3:
        raise RuntimeError(f"verts must be [V, 3], got {tuple(verts.shape)}")
    if faces.dim() != 2 or faces.shape[1] not in (3, 4):
        raise RuntimeError(f"faces must be [F, 3] or [F, 4], got {tuple(faces.shape)}")
    if faces.dtype.is_floating_point:
        raise RuntimeError("faces must hold integer indices")
    v = verts.detach().contiguous()
    f = faces.detach().to(torch.int64).contiguous()
    n = None
    if normals is not None:
        if tuple(normals.shape) != tuple(verts.shape) or normals.dtype != verts.dtype or normals.device != verts.device:
            raise RuntimeError("normals must match verts in shape, dtype and device")
        n = normals.detach().contiguous()
    return v, f, n


def vertex_normals(verts, faces):
    """[V, 3] unit normals: per vertex the sum of its faces' (twice) vector areas,
    normalised; zero for vertices without area.  Deterministic."""
    v, f, _ = _inputs(verts, faces)
    out = torch.empty_like(v)
    with torch.cuda.device(v.device):
        _extractor(v.dtype, v.device).mesh_normals(v, f, out)
    return out


def weld(verts, faces, tol=0.0):
    """Merge vertices with equal positions (tol = 0) or equal rounded positions
    (floor(x / tol + 0.5) per coordinate).  The lowest index of each group stays,
    kept vertices and faces keep their order, faces that collapse are dropped.
    Returns (verts, faces) with faces int64."""
    v, f, _ = _inputs(verts, faces)
    ov = torch.empty_like(v)
    of = torch.empty_like(f)
    with torch.cuda.device(v.device):
        nv, nf = _extractor(v.dtype, v.device).mesh_weld(v, f, tol, ov, of)
    return ov[:nv], of[:nf]


def obj_text(verts, faces, normals=None):
    """The OBJ text as a uint8 CUDA tensor: "v %.8f %.8f %.8f" lines (correctly
    rounded), then "vn" lines when normals are given, then "f" lines with 1-based
    indices ("a//a" with normals)."""
    v, f, n = _inputs(verts, faces, normals)
    with torch.cuda.device(v.device):
        ex = _extractor(v.dtype, v.device)
        size = ex.mesh_obj(v, n, f)
        text = torch.empty(max(size, 1), dtype=torch.uint8, device=v.device)
        ex.mesh_obj(v, n, f, text)
    return text[:size]


def ply_header(n_verts, n_faces, dtype, corners, with_normals):
    t = "float" if dtype == torch.float32 else "double"
    props = ["x", "y", "z"] + (["nx", "ny", "nz"] if with_normals else [])
    lines = ["ply", "format binary_little_endian 1.0", f"element vertex {n_verts}"]
    lines += [f"property {t} {p}" for p in props]
    lines += [f"element face {n_faces}", "property list uchar int vertex_indices", "end_header"]
    return ("\n".join(lines) + "\n").encode("ascii")


def ply_body(verts, faces, normals=None):
    """The binary little-endian PLY body (vertex block, then face block) as a uint8
    CUDA tensor; ply_header gives the header that goes before it."""
    v, f, n = _inputs(verts, faces, normals)
    dt = N.dtype_tag(v.dtype)
    size = int(N.lib().diso_mesh_ply_bytes(dt, v.shape[0], f.shape[0], f.shape[1], int(n is not None)))
    body = torch.empty(max(size, 1), dtype=torch.uint8, device=v.device)
    with torch.cuda.device(v.device):
        _extractor(v.dtype, v.device).mesh_ply(v, n, f, body)
    return body[:size]


def _to_file(path, head, dev_bytes):
    host = torch.empty(dev_bytes.numel(), dtype=torch.uint8, pin_memory=True)
    host.copy_(dev_bytes)
    with open(path, "wb") as fh:
        fh.write(head)
        fh.write(host.numpy().data)


def write_obj(path, verts, faces, normals=None):
    _to_file(path, b"", obj_text(verts, faces, normals))


def write_ply(path, verts, faces, normals=None):
    head = ply_header(verts.shape[0], faces.shape[0], verts.dtype, faces.shape[1], normals is not None)
    _to_file(path, head, ply_body(verts, faces, normals))
