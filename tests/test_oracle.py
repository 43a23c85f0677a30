"""The CPU oracle against the reference's own outputs (golden fixtures produced
by its CUDA extension) and against properties of the surfaces."""
from collections import Counter

import numpy as np
import pytest

from helpers import (assert_faces_equal, assert_grads_close, assert_verts_close, fixture_names, load_fixture)
from oracle import oracle as O

NAMES = fixture_names()


def _method(case):
    return O.MC if case["method"] == "mc" else O.DMC


@pytest.mark.parametrize("name", NAMES)
def test_oracle_forward_matches_reference(name):
    fx = load_fixture(name)
    c = fx["case"]
    v, f, info = O.extract(_method(c), fx["sdf"], fx["deform"], c["iso"], c["normalize"], c["return_quads"],
                           c["dtype"])
    if fx["verts"].shape[0] == 0:
        assert info["empty_guard"] and v.shape == (0, 3) and f.shape == fx["faces"].shape
        assert fx["faces_dtype"] == "torch.int32"
        return
    assert fx["faces_dtype"] == "torch.int64"
    assert_verts_close(v, fx["verts"], c)
    assert_faces_equal(f, fx["faces"], c, fx["verts"])


@pytest.mark.parametrize("name", [n for n in NAMES if load_fixture(n).get("grad_sdf") is not None])
def test_oracle_backward_matches_reference(name):
    fx = load_fixture(name)
    c = fx["case"]
    gs, gd = O.backward(_method(c), fx["sdf"], fx["deform"], fx["weights"], c["iso"], c["normalize"], c["dtype"])
    assert_grads_close(gs, fx["grad_sdf"], c["dtype"], "grad_sdf")
    if fx["deform"] is not None:
        assert_grads_close(gd, fx["grad_deform"], c["dtype"], "grad_deform")


def _sphere(n):
    a = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    return np.sqrt(X * X + Y * Y + Z * Z) - 0.5


def _edge_use(faces):
    c = Counter()
    k = faces.shape[1]
    for t in faces:
        for i in range(k):
            a, b = t[i], t[(i + 1) % k]
            c[(min(a, b), max(a, b))] += 1
    return c


@pytest.mark.parametrize("method,quads", [(O.MC, False), (O.DMC, True), (O.DMC, False)])
def test_closed_manifold_without_deform(method, quads):
    """Without deform both methods give closed 2-manifolds (README: watertight)."""
    rng = np.random.default_rng(5)
    sdf = _sphere(20) + 0.05 * rng.standard_normal((20, 20, 20))
    v, f, _ = O.extract(method, sdf, None, 0.0, True, quads, "float64")
    uses = _edge_use(f)
    assert set(uses.values()) == {2}
    # every vertex is used
    assert np.array_equal(np.unique(f), np.arange(v.shape[0]))


def test_sphere_is_genus_zero():
    sdf = _sphere(32)
    for method in (O.MC, O.DMC):
        v, f, _ = O.extract(method, sdf, None, 0.0, True, method == O.DMC, "float64")
        e = len(_edge_use(f))
        assert v.shape[0] - e + f.shape[0] == 2


def test_mc_vertices_on_crossing_edges():
    rng = np.random.default_rng(3)
    sdf = rng.uniform(-1, 1, (7, 8, 9))
    v, f, _ = O.extract(O.MC, sdf, None, 0.0, False, False, "float64")
    # un-normalised vertices sit on grid edges: two integer coordinates
    frac = np.abs(v - np.round(v)) < 1e-12
    assert (frac.sum(1) >= 2).all()


@pytest.mark.parametrize("method", [O.MC, O.DMC])
def test_oracle_backward_finite_differences(method):
    """Central differences in float64 on points next to crossings."""
    rng = np.random.default_rng(11)
    n = 8
    sdf = _sphere(n) + 0.05 * rng.standard_normal((n, n, n))
    deform = rng.uniform(-0.3, 0.3, (n, n, n, 3))
    v, f, _ = O.extract(method, sdf, deform, 0.0, True, True, "float64")
    w = rng.standard_normal(v.shape)
    gs, gd = O.backward(method, sdf, deform, w, 0.0, True, "float64", exact=True)
    h = 1e-6
    idx = np.argwhere(np.abs(gs) > 0)
    for i in idx[rng.choice(len(idx), 8, replace=False)]:
        i = tuple(i)
        s1, s2 = sdf.copy(), sdf.copy()
        s1[i] += h
        s2[i] -= h
        l1 = (O.extract(method, s1, deform, 0.0, True, True, "float64")[0] * w).sum()
        l2 = (O.extract(method, s2, deform, 0.0, True, True, "float64")[0] * w).sum()
        fd = (l1 - l2) / (2 * h)
        assert abs(fd - gs[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, gs[i])
    j = tuple(np.argwhere(np.abs(gd) > 0)[0])
    d1, d2 = deform.copy(), deform.copy()
    d1[j] += h
    d2[j] -= h
    fd = ((O.extract(method, sdf, d1, 0.0, True, True, "float64")[0] * w).sum()
          - (O.extract(method, sdf, d2, 0.0, True, True, "float64")[0] * w).sum()) / (2 * h)
    assert abs(fd - gd[j]) <= 1e-6 * max(1.0, abs(fd))


@pytest.mark.parametrize("method", [O.MC, O.DMC])
@pytest.mark.parametrize("field", ["sphere", "plane"])
def test_isovalue_gradient_is_minus_the_sdf_gradient_sum(method, field):
    """dL/d(isovalue) = -(sum of dL/dsdf over the grid), the identity behind the
    native isovalue gradient: central differences in the isovalue (float64) against
    the oracle's backward.  The plane crosses the grid's faces, so edges to the pad
    (isovalue + 1, moving with the isovalue) carry vertices too."""
    rng = np.random.default_rng(5)
    n = 10
    a = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    base = _sphere(n) if field == "sphere" else 0.6 * X + 0.3 * Y - 0.2 * Z - 0.1
    sdf = base + 0.03 * rng.standard_normal((n, n, n))
    deform = rng.uniform(-0.3, 0.3, (n, n, n, 3))
    iso, h = 0.02, 1e-6
    v, f, _ = O.extract(method, sdf, deform, iso, True, True, "float64")
    w = rng.standard_normal(v.shape)
    gs, _ = O.backward(method, sdf, deform, w, iso, True, "float64", exact=True)
    lp, fp, _ = O.extract(method, sdf, deform, iso + h, True, True, "float64")
    lm, fm, _ = O.extract(method, sdf, deform, iso - h, True, True, "float64")
    assert np.array_equal(fp, f) and np.array_equal(fm, f)  # the same crossings at both ends
    fd = ((lp * w).sum() - (lm * w).sum()) / (2 * h)
    assert abs(fd + gs.sum()) <= 1e-6 * max(1.0, abs(fd)), (fd, -gs.sum())


def test_empty_guard_when_max_equals_iso():
    sdf = -np.ones((5, 5, 5))
    sdf[2, 2, 2] = 0.0
    v, f, info = O.extract(O.MC, sdf, None, 0.0, True, False, "float32")
    assert info["empty_guard"] and v.shape == (0, 3)


def test_reference_dmc_gradient_differs_only_in_multipatch_cells():
    """The reference's DMC backward gives every patch of a cell the first patch's
    gradient (src/cudualmc.cu:990); on a field with no multi-patch cell both modes agree."""
    rng = np.random.default_rng(2)
    sdf = rng.uniform(-1, 1, (6, 6, 6))
    v, f, _ = O.extract(O.DMC, sdf, None, 0.0, True, True, "float64")
    w = rng.standard_normal(v.shape)
    g_ref, _ = O.backward(O.DMC, sdf, None, w, 0.0, True, "float64")
    g_ex, _ = O.backward(O.DMC, sdf, None, w, 0.0, True, "float64", exact=True)
    assert np.abs(g_ref - g_ex).max() > 0
    s = _sphere(16)
    v, f, _ = O.extract(O.DMC, s, None, 0.0, True, True, "float64")
    w = rng.standard_normal(v.shape)
    a, _ = O.backward(O.DMC, s, None, w, 0.0, True, "float64")
    b, _ = O.backward(O.DMC, s, None, w, 0.0, True, "float64", exact=True)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()
