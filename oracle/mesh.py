"""CPU oracle of the mesh consumers (diso_gb300/mesh.py, diso_mesh_* of the C ABI).

TEST INFRASTRUCTURE ONLY: imported by tests/ and the CPU-baseline leg of
``bench.py``.  The product package never imports it.

numpy restatements of the definitions in include/diso_gb300.h: area-weighted
vertex normals in float64, the lowest-index weld, the OBJ text ("%.8f" through
Python's correctly rounded float formatting) and the binary little-endian PLY
layout.  The reference has no code of its own for these; it calls trimesh's
export (test/example.py:71-73), whose on-disk formats (OBJ, PLY) these follow.
"""
from __future__ import annotations

import numpy as np


def face_normals(verts, faces):
    v = np.asarray(verts, dtype=np.float64)
    f = np.asarray(faces, dtype=np.int64)
    p = v[f]  # [F, k, 3]
    if f.shape[1] == 3:
        a, b = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]
    else:
        a, b = p[:, 2] - p[:, 0], p[:, 3] - p[:, 1]
    return np.cross(a, b)


def vertex_normals(verts, faces):
    """Sum of the face normals (twice the vector areas) around each vertex,
    normalised; zero where the sum is zero.  float64."""
    v = np.asarray(verts)
    f = np.asarray(faces, dtype=np.int64)
    acc = np.zeros((v.shape[0], 3), dtype=np.float64)
    fn = face_normals(v, f)
    for c in range(f.shape[1]):
        np.add.at(acc, f[:, c], fn)
    ln = np.linalg.norm(acc, axis=1, keepdims=True)
    return np.where(ln > 0, acc / np.where(ln > 0, ln, 1.0), 0.0)


def weld_keys(verts, tol):
    v = np.asarray(verts).astype(np.float64)
    if tol > 0:
        return np.floor(v / tol + 0.5).astype(np.int64)
    v = np.where(v == 0.0, 0.0, v)  # -0 counts as +0
    return v.view(np.int64)


def weld(verts, faces, tol=0.0):
    """Vertices with equal keys merge into the lowest index of their group; kept
    vertices and faces keep their order; faces with repeated corners are dropped."""
    v = np.asarray(verts)
    f = np.asarray(faces, dtype=np.int64)
    n = v.shape[0]
    if n == 0:
        return v[:0], f[:0]
    keys = weld_keys(v, tol)
    _, inverse = np.unique(keys, axis=0, return_inverse=True)
    inverse = inverse.reshape(-1)
    lowest = np.full(inverse.max() + 1, n, dtype=np.int64)
    np.minimum.at(lowest, inverse, np.arange(n))
    rep = lowest[inverse]
    keep = rep == np.arange(n)
    new = np.cumsum(keep) - 1
    mapped = new[rep[f]] if f.size else f
    ok = np.ones(f.shape[0], dtype=bool)
    for a in range(f.shape[1]):
        for b in range(a + 1, f.shape[1]):
            ok &= mapped[:, a] != mapped[:, b]
    return v[keep], mapped[ok]


def _fixed8(x):
    return "%.8f" % float(x)


def obj_text(verts, faces, normals=None) -> bytes:
    lines = []
    for p in np.asarray(verts):
        lines.append("v " + " ".join(_fixed8(x) for x in p))
    if normals is not None:
        for p in np.asarray(normals):
            lines.append("vn " + " ".join(_fixed8(x) for x in p))
    for row in np.asarray(faces, dtype=np.int64):
        ids = [str(int(i) + 1) for i in row]
        lines.append("f " + " ".join(f"{i}//{i}" if normals is not None else i for i in ids))
    return "".join(line + "\n" for line in lines).encode("ascii")


def ply_bytes(verts, faces, normals=None) -> bytes:
    v = np.asarray(verts)
    f = np.asarray(faces, dtype=np.int64)
    t = "float" if v.dtype == np.float32 else "double"
    props = ["x", "y", "z"] + (["nx", "ny", "nz"] if normals is not None else [])
    head = ["ply", "format binary_little_endian 1.0", f"element vertex {v.shape[0]}"]
    head += [f"property {t} {p}" for p in props]
    head += [f"element face {f.shape[0]}", "property list uchar int vertex_indices", "end_header"]
    vb = np.concatenate([v, np.asarray(normals, dtype=v.dtype)], axis=1) if normals is not None else v
    vb = np.ascontiguousarray(vb.astype(v.dtype.newbyteorder("<")))
    k = f.shape[1] if f.ndim == 2 else 3
    rec = np.zeros(f.shape[0], dtype=[("n", "u1"), ("i", "<i4", (k,))])
    rec["n"] = k
    rec["i"] = f
    return ("\n".join(head) + "\n").encode("ascii") + vb.tobytes() + rec.tobytes()
