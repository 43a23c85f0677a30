"""Golden cases: seeded inputs on which the reference's own CUDA extension was run.

Each case names the method (MC = DiffMC, DMC = DiffDMC), the dtype, the field,
the grid shape and the call arguments.  ``make_inputs`` rebuilds the inputs from
the seed; the committed fixtures also store them, so tests never depend on the
generator reproducing floats bit for bit across machines.
"""
from __future__ import annotations

import numpy as np

CASES = [
    # the sphere of the reference's example at N=64, plain DiffMC (the first benchmark configuration)
    dict(name="sphere64_mc_f32", method="mc", dtype="float32", field="sphere", shape=(64, 64, 64),
         deform=None, iso=0.0, normalize=True, return_quads=False, loss="sum", seed=0),
    dict(name="sphere64_dmc_f32_quads", method="dmc", dtype="float32", field="sphere", shape=(64, 64, 64),
         deform=None, iso=0.0, normalize=True, return_quads=True, loss="sum", seed=0),
    dict(name="sphere64_dmc_f32_tris", method="dmc", dtype="float32", field="sphere", shape=(64, 64, 64),
         deform=None, iso=0.0, normalize=True, return_quads=False, loss="sum", seed=0),
    # dense random fields: every case code, many ambiguous faces
    dict(name="rand12_mc_f32_def", method="mc", dtype="float32", field="uniform", shape=(12, 12, 12),
         deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=1),
    dict(name="rand12_mc_f64_def", method="mc", dtype="float64", field="uniform", shape=(12, 12, 12),
         deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=2),
    dict(name="rand12_dmc_f32_def_quads", method="dmc", dtype="float32", field="uniform", shape=(12, 12, 12),
         deform=0.45, iso=0.0, normalize=True, return_quads=True, loss="weights", seed=3),
    dict(name="rand12_dmc_f64_def_quads", method="dmc", dtype="float64", field="uniform", shape=(12, 12, 12),
         deform=0.45, iso=0.0, normalize=True, return_quads=True, loss="weights", seed=4),
    dict(name="rand12_dmc_f64_def_tris", method="dmc", dtype="float64", field="uniform", shape=(12, 12, 12),
         deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=5),
    # the round cube of the reference's speed table, small, fp64 with deform
    dict(name="roundcube24_mc_f64_def", method="mc", dtype="float64", field="roundcube", shape=(24, 24, 24),
         deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=8),
    dict(name="roundcube24_dmc_f64_def_tris", method="dmc", dtype="float64", field="roundcube",
         shape=(24, 24, 24), deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=9),
    # non-cubic grids
    dict(name="rand_9x13x6_mc_f64_def", method="mc", dtype="float64", field="uniform", shape=(9, 13, 6),
         deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=10),
    dict(name="rand_9x13x6_dmc_f32_def_quads", method="dmc", dtype="float32", field="uniform", shape=(9, 13, 6),
         deform=0.45, iso=0.0, normalize=True, return_quads=True, loss="weights", seed=11),
    # values exactly at the isovalue (the >= convention decides every code)
    dict(name="ties10_mc_f32", method="mc", dtype="float32", field="ties", shape=(10, 10, 10),
         deform=None, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=12),
    dict(name="ties10_dmc_f32_quads", method="dmc", dtype="float32", field="ties", shape=(10, 10, 10),
         deform=None, iso=0.0, normalize=True, return_quads=True, loss="weights", seed=13),
    # non-zero isovalue, no normalisation
    dict(name="sphere20_mc_f32_iso_nonorm", method="mc", dtype="float32", field="sphere", shape=(20, 20, 20),
         deform=0.3, iso=0.13, normalize=False, return_quads=False, loss="weights", seed=14),
    dict(name="sphere20_dmc_f64_iso_nonorm", method="dmc", dtype="float64", field="sphere", shape=(20, 20, 20),
         deform=0.3, iso=-0.21, normalize=False, return_quads=False, loss="weights", seed=15),
    # empty-surface guard: all above, and max == iso (the guard fires although cells cross)
    dict(name="empty_above_mc_f32", method="mc", dtype="float32", field="const", shape=(6, 6, 6),
         deform=None, iso=0.0, normalize=True, return_quads=False, loss=None, seed=16),
    dict(name="empty_maxiso_dmc_f32", method="dmc", dtype="float32", field="maxiso", shape=(6, 7, 5),
         deform=None, iso=0.0, normalize=True, return_quads=False, loss=None, seed=17),
    # smallest grids
    dict(name="tiny2_mc_f64", method="mc", dtype="float64", field="uniform", shape=(2, 2, 2),
         deform=0.45, iso=0.0, normalize=True, return_quads=False, loss="weights", seed=18),
    dict(name="tiny2_dmc_f64_quads", method="dmc", dtype="float64", field="uniform", shape=(2, 3, 2),
         deform=0.45, iso=0.0, normalize=True, return_quads=True, loss="weights", seed=19),
]


def grid_coords(shape, dtype):
    """linspace(-1, 1, n) per axis, indexed [x, y, z] as in the reference's example."""
    axes = [np.linspace(-1.0, 1.0, n) for n in shape]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    return np.stack([X, Y, Z], -1).astype(dtype)


def make_inputs(case):
    """(sdf, deform or None) for a case, seeded."""
    dt = np.dtype(case["dtype"])
    rng = np.random.default_rng(case["seed"])
    shape = tuple(case["shape"])
    f = case["field"]
    if f == "sphere":
        p = grid_coords(shape, np.float64)
        sdf = np.linalg.norm(p, axis=-1) - 0.5
    elif f == "roundcube":
        p = grid_coords(shape, np.float64)
        q = np.maximum(np.abs(p) - 0.5, 0.0)
        sdf = np.linalg.norm(q, axis=-1) - 0.1
    elif f == "uniform":
        sdf = rng.uniform(-1.0, 1.0, shape)
    elif f == "ties":
        sdf = rng.integers(-1, 2, shape) * 0.5
    elif f == "const":
        sdf = np.ones(shape)
    elif f == "maxiso":
        sdf = -rng.uniform(0.1, 1.0, shape)
        sdf[1, 2, 3] = 0.0
    else:
        raise ValueError(f)
    sdf = sdf.astype(dt)
    deform = None
    if case["deform"]:
        a = case["deform"]
        deform = rng.uniform(-a, a, shape + (3,)).astype(dt)
    return sdf, deform


def loss_weights(case, nverts):
    """Fixed N(0,1) weights of the loss sum(verts * w)."""
    rng = np.random.default_rng(1000 + case["seed"])
    return rng.standard_normal((nverts, 3)).astype(case["dtype"])
