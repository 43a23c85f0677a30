"""Shared test helpers: golden fixtures, the reference's tolerances and the
comparisons used by both the oracle tests (CPU) and the CUDA parity tests (GPU).

Tolerances (the bar for this path):
* case codes, face index lists and vertex counts: exact;
* vertices: within 1e-6 of the grid extent in float32, 1e-12 in float64
  (extent = 1 with normalize, dim - 1 without);
* gradients: max |a - b| <= 1e-5 * max |b| in float32 (1e-10 in float64) against
  the reference's own outputs.  Against the float64 oracle a float32 result also
  carries the reference's rounding of p = X + deform at magnitude X (up to
  N * 2^-24 on p1 - p0), so that bound is scaled by max(1, N / 32);
* DMC quad -> triangle split: the same choice for every quad except true
  near-ties, |max_cos1 - max_cos2| < 1e-5 (float32) / 1e-12 (float64) as
  evaluated in float64 on the reference's vertices.
"""
from __future__ import annotations

import glob
import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
FIXTURES = os.path.join(GOLDEN, "fixtures")
if GOLDEN not in sys.path:
    sys.path.insert(0, GOLDEN)

from cases import loss_weights, make_inputs  # noqa: E402

VERT_TOL = {"float32": 1e-6, "float64": 1e-12}
GRAD_RTOL = {"float32": 1e-5, "float64": 1e-10}
SPLIT_TIE = {"float32": 1e-5, "float64": 1e-12}


def fixture_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(FIXTURES, "*.npz")))


def load_fixture(name):
    d = dict(np.load(os.path.join(FIXTURES, name + ".npz")))
    case = json.loads(str(d["meta"]))
    fx = dict(case=case, sdf=d["sdf"], deform=d.get("deform"), verts=d["verts"],
              faces=d["faces"].astype(np.int64), faces_dtype=str(d["faces_dtype"]))
    shape = d["sdf"].shape
    if "grad_sdf_idx" in d:
        g = np.zeros(int(np.prod(shape)), d["grad_sdf_val"].dtype)
        g[d["grad_sdf_idx"]] = d["grad_sdf_val"]
        fx["grad_sdf"] = g.reshape(shape)
        if "grad_deform_idx" in d:
            gd = np.zeros(int(np.prod(shape)) * 3, d["grad_deform_val"].dtype)
            gd[d["grad_deform_idx"]] = d["grad_deform_val"]
            fx["grad_deform"] = gd.reshape(shape + (3,))
    if case["loss"] == "weights" and fx["verts"].shape[0]:
        w = loss_weights(case, fx["verts"].shape[0])
        if "weights_sha256" in d:
            assert hashlib.sha256(w.tobytes()).hexdigest() == str(d["weights_sha256"]), "loss weights changed"
        fx["weights"] = w
    elif case["loss"] == "sum":
        fx["weights"] = np.ones_like(fx["verts"])
    return fx


def extent(case):
    return 1.0 if case["normalize"] else float(max(case["shape"]) - 1)


def assert_verts_close(v, v_ref, case):
    assert v.shape == v_ref.shape, (v.shape, v_ref.shape)
    if v.size == 0:
        return
    tol = VERT_TOL[case["dtype"]] * extent(case)
    a, b = v.astype(np.float64), v_ref.astype(np.float64)
    # a unit-length axis with normalize divides by dim - 1 = 0 (as the reference does):
    # the non-finite entries must then agree exactly
    fa, fb = np.isfinite(a), np.isfinite(b)
    assert np.array_equal(fa, fb), "non-finite vertex coordinates differ"
    assert np.array_equal(a[~fa], b[~fb], equal_nan=True), "non-finite vertex coordinates differ"
    if fa.any():
        err = np.abs(a[fa] - b[fb]).max()
        assert err <= tol, f"vertex error {err:.3e} > {tol:.1e}"


def oracle_grad_rtol(dtype, shape):
    """Gradient tolerance of a float32 / float64 result against the float64 oracle."""
    return GRAD_RTOL[dtype] * (max(1.0, max(shape) / 32.0) if dtype == "float32" else 1.0)


def assert_grads_close(g, g_ref, dtype, what="grad", rtol=None):
    assert g.shape == g_ref.shape
    fa, fb = np.isfinite(g), np.isfinite(g_ref)
    assert np.array_equal(fa, fb), f"{what}: non-finite entries differ"
    if not fa.all():
        assert np.array_equal(g[~fa], g_ref[~fb], equal_nan=True), f"{what}: non-finite entries differ"
        g, g_ref = np.where(fa, g, 0), np.where(fb, g_ref, 0)
    scale = np.abs(g_ref).max()
    if scale == 0:
        assert np.abs(g).max() == 0, f"{what}: expected all zeros"
        return
    rtol = GRAD_RTOL[dtype] if rtol is None else rtol
    err = np.abs(g.astype(np.float64) - g_ref.astype(np.float64)).max()
    assert err <= rtol * scale, f"{what}: max error {err:.3e} > {rtol:.1e} * {scale:.3e}"


def _tri_max_cos(V, a, b, c):
    p = [V[a], V[b], V[c]]
    m = None
    for i in range(3):
        o, u, w = p[i], p[(i + 1) % 3], p[(i + 2) % 3]
        e1, e2 = u - o, w - o
        n1 = e1 / max(np.linalg.norm(e1), 1e-12)
        n2 = e2 / max(np.linalg.norm(e2), 1e-12)
        cs = float(n1 @ n2)
        m = cs if m is None else max(m, cs)
    return m


def split_margin(V, q):
    """|max_cos1 - max_cos2| of a quad in float64."""
    V = V.astype(np.float64)
    m1 = max(_tri_max_cos(V, q[0], q[1], q[3]), _tri_max_cos(V, q[1], q[2], q[3]))
    m2 = max(_tri_max_cos(V, q[0], q[1], q[2]), _tri_max_cos(V, q[0], q[2], q[3]))
    return abs(m1 - m2)


def decode_split(tris):
    """Triangle pairs of a quad split -> list of (quad tuple, config)."""
    out = []
    t = tris.reshape(-1, 2, 3)
    for a, b in t:
        if a[1] == b[0] and a[2] == b[2]:  # (q0,q1,q3),(q1,q2,q3)
            out.append(((a[0], a[1], b[1], a[2]), 1))
        elif a[0] == b[0] and a[2] == b[1]:  # (q0,q1,q2),(q0,q2,q3)
            out.append(((a[0], a[1], a[2], b[2]), 2))
        else:
            raise AssertionError(f"not a quad split pair: {a} {b}")
    return out


def assert_faces_equal(f, f_ref, case, verts_ref=None):
    """Exact equality; for DMC triangles allow split flips only on near-ties."""
    assert f.shape == f_ref.shape, (f.shape, f_ref.shape)
    if np.array_equal(f, f_ref):
        return
    if case["method"] == "dmc" and not case["return_quads"] and verts_ref is not None:
        mine, ref = decode_split(f), decode_split(f_ref)
        dm, dr = dict(mine), dict(ref)
        assert len(dm) == len(mine) and len(dr) == len(ref), "repeated quads"
        assert set(dm) == set(dr), "different quad sets"
        tie = SPLIT_TIE[case["dtype"]]
        flips = [q for q in dr if dm[q] != dr[q]]
        for q in flips:
            marg = split_margin(verts_ref, q)
            assert marg < tie, f"split of quad {q} differs with margin {marg:.3e}"
        # order: config-1 quads first in quad order, then config-2 quads
        return
    bad = np.nonzero((f != f_ref).any(1))[0]
    raise AssertionError(f"{len(bad)} faces differ, first at {bad[:5]}: {f[bad[:3]]} vs {f_ref[bad[:3]]}")
