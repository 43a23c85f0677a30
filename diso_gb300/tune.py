"""Autotuner of the extractor's launch widths.

The free parameters of the kernels' launches (persistent CTAs per SM of the
count, the emit, the backward passes, the zero fills, the batches, and the share
of the gradient zeros the stored mode's count writes; diso_tune_set) change no
output: every kernel gives the same bits for any width.  Their best values
depend on the GPU, the method, the dtype, the grid size and the backward mode, so
they are found by timing, once per (GPU, method, dtype, size bucket, mode), on a
synthetic field of the caller's size (a noisy union of spheres with a deform, the
kind of surface the benchmark extracts), and cached on disk:

    from diso_gb300 import DiffDMC, tune
    mod = DiffDMC(torch.float32, recompute=True)
    tune.tune_module(mod, (512, 512, 512))          # times candidates, caches, applies
    # later processes: tune.tune_module(mod, shape) applies the cached winner at once

The search is coordinate descent over the parameters that the mode's kernels
read, starting from the defaults, each candidate timed with CUDA events over a
few forward + backward steps.  The reference fixes its block size (BLOCK_SIZE 512,
src/cumc.cu:93) and has nothing to tune.

The cache file is $DISO_TUNE_CACHE, else ~/.cache/diso_gb300/tune.json.
"""
from __future__ import annotations

import json
import os
import threading

import torch

from . import _native as N

# candidates per parameter; 0 is the library's default
CANDIDATES = {
    "count_ctas": [0, 1],
    "emit_ctas": [0, 2, 3],
    "gather_ctas": [0, 2, 3],
    "fused_ctas": [0, 2],
    "zero_ctas": [0, 1, 4],
    "edge_ctas": [0, 4, 16],
    "batch_ctas": [0, 2, 8],
    "zero_share": [0, 250, 450],
}
# the parameters each workload's kernels read
MODE_PARAMS = {
    "stored": ["count_ctas", "emit_ctas", "gather_ctas", "edge_ctas", "zero_share"],
    "recompute": ["count_ctas", "emit_ctas", "fused_ctas", "zero_ctas"],
    "batch": ["batch_ctas", "gather_ctas", "edge_ctas", "zero_ctas"],
}

_lock = threading.Lock()


def cache_path() -> str:
    return os.environ.get("DISO_TUNE_CACHE") or os.path.join(os.path.expanduser("~"), ".cache", "diso_gb300",
                                                             "tune.json")


def bucket(shape) -> str:
    """Size bucket of a grid: the power of two at or above its largest side (>= 32)."""
    n = max(int(x) for x in shape)
    b = 32
    while b < n:
        b *= 2
    return f"n{b}"


def key(device, method: int, dtype: torch.dtype, shape_bucket: str, mode: str) -> str:
    name = torch.cuda.get_device_name(device) if torch.cuda.is_available() else "cpu"
    return "|".join([name, "mc" if method == N.MC else "dmc", str(dtype).replace("torch.", ""), shape_bucket, mode])


def load_cache(path=None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) else {}
    except (OSError, ValueError):
        return {}


def store(k: str, entry: dict, path=None):
    """Add one entry to the cache file (read, update, write to a temporary, rename)."""
    path = path or cache_path()
    with _lock:
        data = load_cache(path)
        data[k] = entry
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = f"{path}.{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def coordinate_descent(params, candidates, measure, start=None):
    """Minimise measure(setting) one parameter at a time, in order, over its
    candidates, keeping the others at their best so far.  Returns (best setting,
    its time, {str(setting): time} of every setting measured)."""
    best = dict(start or {p: 0 for p in params})
    seen = {}

    def timed(s):
        k = json.dumps(s, sort_keys=True)
        if k not in seen:
            seen[k] = measure(dict(s))
        return seen[k]

    best_t = timed(best)
    for p in params:
        for v in candidates[p]:
            if v == best[p]:
                continue
            trial = dict(best)
            trial[p] = v
            t = timed(trial)
            if t < best_t:
                best, best_t = trial, t
    return best, best_t, seen


def synthetic_grid(shape, device, dtype, seed=5):
    """A noisy union of 16 spheres on [-1, 1]^3 with a deform U(-0.3, 0.3): dense
    crossings near a large surface, like the benchmark's field."""
    g = torch.Generator().manual_seed(seed)
    c = (torch.rand(16, 3, generator=g, dtype=torch.float64) * 1.6 - 0.8).tolist()
    r = (torch.rand(16, generator=g, dtype=torch.float64) * 0.25 + 0.05).tolist()
    axes = [torch.linspace(-1, 1, n, device=device, dtype=dtype) for n in shape]
    X, Y, Z = axes[0].view(-1, 1, 1), axes[1].view(1, -1, 1), axes[2].view(1, 1, -1)
    s = None
    for (cx, cy, cz), rr in zip(c, r):
        d = torch.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) - rr
        s = d if s is None else torch.minimum(s, d)
    gg = torch.Generator(device=device).manual_seed(seed)
    s = (s + 0.01 * torch.randn(tuple(shape), device=device, dtype=dtype, generator=gg)).contiguous()
    dfm = (torch.rand(tuple(shape) + (3,), device=device, dtype=dtype, generator=gg) * 0.6 - 0.3).contiguous()
    return s, dfm


def time_module(mod, sdf, deform, steps=5, warmup=2, **kw):
    """Milliseconds per forward + backward step of `mod` on the resident inputs."""
    s = sdf.clone().requires_grad_(True)
    d = deform.clone().requires_grad_(True)
    w = None

    def step():
        nonlocal w
        s.grad = None
        d.grad = None
        v, _ = mod(s, d, **kw)
        if w is None or w.shape != v.shape:
            w = torch.randn(v.shape, dtype=v.dtype, device=v.device)
        (v * w).sum().backward()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        step()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def tune_module(mod, shape, retune=False, steps=5, path=None) -> dict:
    """Launch widths for DiffMC / DiffDMC `mod` on grids of `shape`: the cached
    winner of this (GPU, method, dtype, size bucket, mode), else found by timing
    (and cached); applied to the module's extractor.  Returns the cache entry."""
    ex = mod._ex
    device = torch.device("cuda", torch.cuda.current_device())
    mode = "recompute" if getattr(mod, "recompute", False) else "stored"
    k = key(device, ex.method, ex.dtype, bucket(shape), mode)
    entry = None if retune else load_cache(path).get(k)
    if entry is None:
        sdf, dfm = synthetic_grid(shape, device, ex.dtype)
        kw = {"return_quads": True} if ex.method == N.DMC else {}

        def measure(setting):
            ex.set_launch(setting)
            return time_module(mod, sdf, dfm, steps=steps, **kw)

        params = MODE_PARAMS[mode]
        best, best_t, seen = coordinate_descent(params, CANDIDATES, measure)
        default_t = seen[json.dumps({p: 0 for p in params}, sort_keys=True)]
        entry = {"params": best, "ms": best_t, "default_ms": default_t, "trials": len(seen),
                 "shape": list(shape)}
        store(k, entry, path)
        del sdf, dfm
    ex.set_launch(entry["params"])
    return entry


def tune_plan(plan, retune=False, steps=5, path=None) -> dict:
    """Launch widths of a BatchPlan's eager run (its extractor), found by timing
    plan.run on the plan's current contents, cached per (GPU, method, dtype, batch
    of the plan's largest grid, "batch") and applied; capture the plan afterwards."""
    ex = plan.bx.ex
    device = torch.device("cuda", torch.cuda.current_device())
    biggest = max(plan.shapes, key=lambda s: s[0] * s[1] * s[2])
    k = key(device, ex.method, ex.dtype, f"{len(plan.shapes)}x{bucket(biggest)}", "batch")
    entry = None if retune else load_cache(path).get(k)
    if entry is None:
        def measure(setting):
            ex.set_launch(setting)
            for _ in range(2):
                plan.run()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(steps):
                plan.run()
            b.record()
            torch.cuda.synchronize()
            return a.elapsed_time(b) / steps

        params = MODE_PARAMS["batch"]
        best, best_t, seen = coordinate_descent(params, CANDIDATES, measure)
        default_t = seen[json.dumps({p: 0 for p in params}, sort_keys=True)]
        entry = {"params": best, "ms": best_t, "default_ms": default_t, "trials": len(seen)}
        store(k, entry, path)
    ex.set_launch(entry["params"])
    return entry
