#!/usr/bin/env python
"""Benchmark: forward + backward of DiffDMC on a 512^3 float32 SDF, in grids/s.

Workload (one "step" = one extraction and its backward over one grid): 512^3
float32 SDF, the minimum of 16 seeded spheres (centres U(-0.8, 0.8)^3, radii
U(0.05, 0.3)) plus 0.01 * N(0, 1) noise, deform U(-0.45, 0.45) [512,512,512,3],
DiffDMC with return_quads=True and normalize=True, loss = sum(verts * w) with
fixed seeded N(0, 1) weights.  Inputs (2.15 GB) are larger than L2 (129 MB), so
no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 512]

Prints one JSON line.  ``value`` is device-resident throughput; ``e2e`` repeats
the step through the same public API with the inputs copied from pinned host
memory each step and the loss read back (the inputs double-buffered: the next
step's copy runs on a second stream while the current step computes).  ``--impl reference`` times the CPU
implementation of the same path (the reference has no CPU code; the project's
OpenMP FP64 restatement in oracle/ stands in) on bounded samples of the grid.
Under torchrun each rank runs its own replica of the workload (no collective on
the data path); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

SEED = 2
DEFORM = 0.45


def metric_name(n):
    return f"fwd+bwd grids/s @{n}^3 (DiffDMC, fp32, deform, return_quads)"


def spheres_field(n, device, dtype=torch.float32, seed=SEED):
    g = torch.Generator().manual_seed(seed)
    c = (torch.rand(16, 3, generator=g, dtype=torch.float64) * 1.6 - 0.8).tolist()
    r = (torch.rand(16, generator=g, dtype=torch.float64) * 0.25 + 0.05).tolist()
    lin = torch.linspace(-1, 1, n, device=device, dtype=dtype)
    X, Y, Z = lin.view(n, 1, 1), lin.view(1, n, 1), lin.view(1, 1, n)
    s = None
    for (cx, cy, cz), rr in zip(c, r):
        d = torch.sqrt((X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2) - rr
        s = d if s is None else torch.minimum(s, d)
    gg = torch.Generator(device=device).manual_seed(seed)
    s = s + 0.01 * torch.randn(n, n, n, device=device, dtype=dtype, generator=gg)
    return s.contiguous()


def deform_field(n, device, dtype=torch.float32, seed=SEED):
    gg = torch.Generator(device=device).manual_seed(seed + 100)
    return (torch.rand(n, n, n, 3, device=device, dtype=dtype, generator=gg) * (2 * DEFORM) - DEFORM).contiguous()


def loss_weights(nv, device, dtype):
    g = torch.Generator(device=device).manual_seed(SEED + 200)
    return torch.randn(nv, 3, device=device, dtype=dtype, generator=g)


# ----------------------------------------------------------------------------- uneven grids
def object_field(shape, kind, rng, device, dtype=torch.float32, noise=0.02):
    """Sphere (radius U(0.3, 0.7)) or rounded box (half-extent U(0.3, 0.6), radius 0.1)
    on linspace(-1, 1) axes, plus N(0, noise) noise; `rng` is a numpy Generator."""
    axes = [torch.linspace(-1, 1, n, device=device, dtype=dtype) for n in shape]
    X, Y, Z = axes[0].view(-1, 1, 1), axes[1].view(1, -1, 1), axes[2].view(1, 1, -1)
    if kind == "sphere":
        s = torch.sqrt(X * X + Y * Y + Z * Z) - float(rng.uniform(0.3, 0.7))
    else:
        h = float(rng.uniform(0.3, 0.6))
        q = torch.stack(torch.broadcast_tensors((X.abs() - h).clamp_min(0), (Y.abs() - h).clamp_min(0),
                                                (Z.abs() - h).clamp_min(0)), -1)
        s = q.norm(dim=-1) - 0.1
    g = torch.Generator(device=device).manual_seed(int(rng.integers(1 << 31)))
    return (s + noise * torch.randn(shape, device=device, dtype=dtype, generator=g)).contiguous()


def uneven_batch(ngrids=64, seed=1, device="cuda", dtype=torch.float32, deform=0.3):
    """The batched workload: N log-uniform in [32, 256], sphere or rounded box + noise, deform U(-0.3, 0.3)."""
    rng = np.random.default_rng(seed)
    sdfs, defs = [], []
    for _ in range(ngrids):
        n = int(round(float(np.exp(rng.uniform(np.log(32), np.log(256))))))
        kind = "sphere" if rng.random() < 0.5 else "box"
        sdfs.append(object_field((n, n, n), kind, rng, device, dtype))
        g = torch.Generator(device=device).manual_seed(int(rng.integers(1 << 31)))
        defs.append((torch.rand((n, n, n, 3), device=device, dtype=dtype, generator=g) * 2 * deform - deform).contiguous())
    return sdfs, defs


def request_inputs(seed, shape, kind, deform=0.3, dtype=torch.float32):
    """Device inputs of one served request, rebuilt identically from its seed:
    (sdf, deform, dL/dverts generator)."""

    def make(device):
        rng = np.random.default_rng(seed)
        if kind == "random":
            g = torch.Generator(device=device).manual_seed(seed)
            sdf = torch.rand(shape, device=device, dtype=dtype, generator=g) * 2 - 1
        else:
            sdf = object_field(shape, kind, rng, device, dtype)
        g = torch.Generator(device=device).manual_seed(seed + 1)
        dfm = (torch.rand(shape + (3,), device=device, dtype=dtype, generator=g) * 2 * deform - deform).contiguous()

        def grad(nv):
            gg = torch.Generator(device=device).manual_seed(seed + 2)
            return torch.randn((nv, 3), device=device, dtype=dtype, generator=gg)

        return sdf, dfm, grad

    return make


class InputPool:
    """Device-resident payloads of served requests: per (N, kind) a few grids with
    their deforms, generated once before serving (a request names one by its seed),
    and one buffer of N(0, 1) loss gradients that every request slices.  Requests
    thus arrive with their data already on the device, as in a server whose clients
    upload grids, and neither the server nor the per-request baseline spends its
    measured time synthesising inputs.  Each request gets its own views (its own
    autograd leaves); the payloads are only read."""

    def __init__(self, device, variants=4, max_verts=150_000_000):
        self.device, self.variants = device, variants
        self.grids = {}
        self.gv = torch.randn((max_verts, 3), device=device, dtype=torch.float32,
                              generator=torch.Generator(device=device).manual_seed(SEED + 300))

    def get(self, n, kind, v):
        key = (n, kind, v)
        if key not in self.grids:
            sdf, dfm, _ = request_inputs(1000 * n + 10 * v + ["random", "sphere", "box"].index(kind),
                                         (n, n, n), kind)(self.device)
            self.grids[key] = (sdf, dfm)
        sdf, dfm = self.grids[key]
        return sdf.detach(), dfm.detach(), self.grad

    def grad(self, nv):
        if nv > self.gv.shape[0]:
            raise RuntimeError(f"{nv} vertices exceed the gradient pool ({self.gv.shape[0]})")
        return self.gv[:nv]

    def warm(self):
        for n in (64, 128, 256, 384):
            for kind in ("random", "sphere", "box"):
                for v in range(self.variants):
                    self.get(n, kind, v)
        torch.cuda.synchronize(self.device)


def served_trace(nreq=2000, rate=2000.0, seed=3, pool=None):
    """Poisson arrivals; N in {64,128,256,384} at {.4,.3,.2,.1}; MC / DMC 50/50;
    U(-1,1) random fields 30%, sphere / rounded box 70%; deform U(-0.3, 0.3).  With
    a pool the requests' payloads are its device-resident grids; without one each
    request generates its own on the device."""
    from diso_gb300.serve import Request, estimate_bytes

    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(nreq):
        t += float(rng.exponential(1.0 / rate))
        n = int(rng.choice([64, 128, 256, 384], p=[0.4, 0.3, 0.2, 0.1]))
        method = int(rng.integers(2))
        u = rng.random()
        kind = "random" if u < 0.3 else ("sphere" if u < 0.65 else "box")
        shape = (n, n, n)
        rs = int(rng.integers(1 << 30))
        if pool is not None:
            make = (lambda n_, k_, v_: (lambda dev: pool.get(n_, k_, v_)))(n, kind, rs % pool.variants)
        else:
            make = request_inputs(rs, shape, kind)
        req = Request(rid=i, method=method, shape=shape, arrival=t, make_inputs=make,
                      est_bytes=estimate_bytes(shape, dense=kind == "random"))
        req.kind = kind
        out.append(req)
    return out


def device_bound(trace, pool, device, reps=3):
    """grids/s of the trace if the GPU ran nothing but the plain per-request call's
    kernels back to back: per (N, kind, method) the extractor's kernel time of one
    request (CUDA events around every launch), summed over the trace.  The plain loop
    cannot serve the trace faster than this; the server can, as far as its batched
    kernels do less device work per grid."""
    from diso_gb300 import _native as N
    from diso_gb300.extraction import extract

    ex = {m: N.Extractor(m, torch.float32) for m in (N.MC, N.DMC)}
    per = {}
    for key in sorted({(r.shape[0], r.kind, r.method) for r in trace}):
        n, kind, m = key
        e = ex[m]

        def one():
            sdf, dfm, grad = pool.get(n, kind, 0)
            sdf.requires_grad_(True)
            dfm.requires_grad_(True)
            v, _ = extract(e, sdf, dfm, 0.0, True, True)
            torch.autograd.backward(v, grad(v.shape[0]))

        one()
        torch.cuda.synchronize()
        e.timing(True)
        for _ in range(reps):
            one()
        torch.cuda.synchronize()
        per[key] = sum(ms for _, ms in e.timing_read().values()) / reps
        e.timing(False)
    total_ms = sum(per[(r.shape[0], r.kind, r.method)] for r in trace)
    return len(trace) / (total_ms * 1e-3), per


def run_batched(device, method, steps=10, warmup=3, ngrids=64):
    """grids/s of a plain per-grid loop against one batched launch per phase (eager and
    CUDA-graph replay), forward + backward, on the uneven batch."""
    from diso_gb300 import BatchPlan, DiffDMC, DiffMC

    sdfs, defs = uneven_batch(ngrids, device=device)
    ext = DiffMC(torch.float32) if method == 0 else DiffDMC(torch.float32)
    ins = [(s.clone().requires_grad_(True), d.clone().requires_grad_(True)) for s, d in zip(sdfs, defs)]
    kw = {} if method == 0 else {"return_quads": True}
    ws = [loss_weights(ext(s, d, **kw)[0].shape[0], device, torch.float32) for s, d in ins]

    def loop():
        for (s, d), w in zip(ins, ws):
            s.grad = None
            d.grad = None
            v, _ = ext(s, d, **kw)
            torch.autograd.backward(v, w)

    def timed(fn, k):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(k):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / k

    ms_loop = timed(loop, steps)
    plan = BatchPlan(method, torch.float32, [tuple(s.shape) for s in sdfs], deform=True)
    for i, (s, d) in enumerate(zip(sdfs, defs)):
        plan.sdf[i].copy_(s)
        plan.deform[i].copy_(d)
    nv, _ = plan.size_outputs()
    plan.grad_verts[:nv].copy_(torch.cat(ws))
    from diso_gb300 import tune

    tuned = tune.tune_plan(plan)
    ms_eager = timed(plan.run, steps)
    plan.capture()
    ms_graph = timed(plan.replay, steps)
    plan.results()
    return {"grids": ngrids, "loop_grids_s": ngrids / (ms_loop * 1e-3), "batched_grids_s": ngrids / (ms_eager * 1e-3),
            "graph_grids_s": ngrids / (ms_graph * 1e-3), "speedup_vs_loop": ms_loop / ms_graph,
            "launch": tuned["params"],
            "ms_loop": ms_loop, "ms_graph": ms_graph}


def run_mesh(device, n=512, steps=5, warmup=2, cpu_sample=100000):
    """The mesh consumers on the benchmark's DMC mesh (quads): device times of vertex
    normals, weld, OBJ text and PLY body (CUDA events), the files written through the
    public calls (host wall time: device work, copy to pinned memory, file write), and
    the CPU oracle on a sample of the mesh, scaled to the whole."""
    import tempfile

    from diso_gb300 import DiffDMC, mesh

    sdf = spheres_field(n, device)
    deform = deform_field(n, device)
    with torch.no_grad():
        v, f = DiffDMC(torch.float32)(sdf, deform, return_quads=True)
    del sdf, deform
    nv, nf = v.shape[0], f.shape[0]
    nrm = mesh.vertex_normals(v, f)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, out

    res = {"mesh": f"DMC quads of the {n}^3 benchmark grid", "verts": nv, "quads": nf}
    ms, _ = timed(lambda: mesh.vertex_normals(v, f))
    # faces twice (max pass, sum pass) with their corners' vertices, 24 B of sums per
    # corner (read + write), normals out
    by = 2 * nf * (4 * 8 + 4 * 12) + nf * 4 * 24 + nv * 12
    res["normals_ms"] = ms
    res["normals_gbs"] = by / (ms * 1e-3) / 1e9
    ms, (wv, wf) = timed(lambda: mesh.weld(v, f))
    res["weld_ms"], res["weld_verts"], res["weld_quads"] = ms, wv.shape[0], wf.shape[0]
    ms, text = timed(lambda: mesh.obj_text(v, f, nrm))
    res["obj_ms"], res["obj_bytes"] = ms, text.numel()
    res["obj_gbs"] = text.numel() / (ms * 1e-3) / 1e9
    ms, body = timed(lambda: mesh.ply_body(v, f, nrm))
    res["ply_ms"], res["ply_bytes"] = ms, body.numel()
    del text, body
    with tempfile.TemporaryDirectory() as tmp:
        for kind, fn in (("obj", mesh.write_obj), ("ply", mesh.write_ply)):
            path = os.path.join(tmp, "mesh." + kind)
            fn(path, v, f, nrm)
            t0 = time.perf_counter()
            fn(path, v, f, nrm)
            res[f"write_{kind}_ms"] = (time.perf_counter() - t0) * 1e3
    # the CPU oracle (numpy normals, Python OBJ formatting) on the first cpu_sample
    # vertices and the faces among them, scaled by the vertex count
    from oracle import mesh as M

    k = min(cpu_sample, nv)
    hv, hf = v[:k].cpu().numpy(), f.cpu().numpy()
    hf = hf[(hf < k).all(axis=1)]
    hn = M.vertex_normals(hv, hf)
    t0 = time.perf_counter()
    M.vertex_normals(hv, hf)
    t1 = time.perf_counter()
    M.obj_text(hv, hf, hn)
    t2 = time.perf_counter()
    res["cpu_baseline"] = {"normals_ms": (t1 - t0) * 1e3 * nv / k, "obj_ms": (t2 - t1) * 1e3 * nv / k, "cores": 1,
                           "kind": "port", "sample": f"first {k} vertices and their {hf.shape[0]} quads, scaled"}
    return res


def run_field(device, n=512, steps=10, warmup=3):
    """The benchmark's 16 spheres (without the noise, which no closed form has) as an
    evaluated field on [-1, 1]^3 at n^3: the fused forward (no dense grid) against
    materialising the grid and running the dense forward, DiffDMC with quads, no
    gradients.  Both give the same mesh (tests/test_gpu_fields.py)."""
    from diso_gb300 import DiffDMC, SphereUnion

    g = torch.Generator().manual_seed(SEED)
    c = torch.rand(16, 3, generator=g, dtype=torch.float64) * 1.6 - 0.8
    r = torch.rand(16, generator=g, dtype=torch.float64) * 0.25 + 0.05
    field = SphereUnion(c.to(device, torch.float32), r.to(device, torch.float32))
    mod = DiffDMC(torch.float32)

    def dense():
        with torch.no_grad():
            return mod(field.materialize((n, n, n)), return_quads=True)

    def fused():
        return mod.forward_field(field, (n, n, n), return_quads=True)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, out

    ms_d, (vd, qd) = timed(dense)
    ms_f, (vf, qf) = timed(fused)
    return {"field": f"16 spheres on [-1,1]^3 at {n}^3, DiffDMC quads, forward", "verts": vf.shape[0],
            "quads": qf.shape[0], "same_mesh": bool(torch.equal(vd, vf) and torch.equal(qd, qf)),
            "dense_ms": ms_d, "fused_ms": ms_f, "speedup": ms_d / ms_f}


def sphere_band(n, device, dtype=torch.float32, seed=SEED, halo=12.0, deform=True):
    """The benchmark's 16 spheres (without the noise) as a narrow band at n^3 on
    [-1, 1]^3, built brick by brick without a dense grid: bricks whose centre lies
    within `halo` grid steps of the surface are present (the union's distance is
    1-Lipschitz, so the others, more than their half diagonal from it, lie on one side
    and are tagged by it); deform U(-0.45, 0.45) at the bricks' points."""
    from diso_gb300 import BrickGrid

    g = torch.Generator().manual_seed(seed)
    c = (torch.rand(16, 3, generator=g, dtype=torch.float64) * 1.6 - 0.8).to(device)
    r = (torch.rand(16, generator=g, dtype=torch.float64) * 0.25 + 0.05).to(device)
    step = 2.0 / (n - 1)
    nb = (n + 7) // 8

    def dist(p):  # p [..., 3] float64 -> min_k |p - c_k| - r_k
        out = None
        for k in range(16):
            d = (p - c[k]).norm(dim=-1) - r[k]
            out = d if out is None else torch.minimum(out, d)
        return out

    ax = -1.0 + (torch.arange(nb, device=device, dtype=torch.float64) * 8 + 3.5) * step
    dc = torch.empty((nb, nb, nb), dtype=torch.float64, device=device)
    for i in range(nb):
        P = torch.stack(torch.meshgrid(ax[i:i + 1], ax, ax, indexing="ij"), -1)
        dc[i] = dist(P)[0]
    present = dc.abs() <= halo * step
    k = int(present.sum())
    index = torch.where(dc > 0, -1, -2).to(torch.int32)
    index[present] = torch.arange(k, dtype=torch.int32, device=device)
    bricks = torch.nonzero(present)  # slot order: x-major, as the index numbers them
    lr = torch.arange(8, device=device, dtype=torch.float64)
    loc = torch.stack(torch.meshgrid(lr, lr, lr, indexing="ij"), -1).reshape(1, 512, 3)
    values = torch.empty((k, 8, 8, 8), dtype=dtype, device=device)
    for a in range(0, k, 32768):
        b = bricks[a:a + 32768].to(torch.float64)
        P = -1.0 + (b[:, None, :] * 8 + loc) * step
        values[a:a + 32768] = dist(P).reshape(-1, 8, 8, 8).to(dtype)
    dfm = None
    if deform:
        gg = torch.Generator(device=device).manual_seed(seed + 100)
        dfm = torch.rand((k, 8, 8, 8, 3), device=device, dtype=dtype, generator=gg) * (2 * DEFORM) - DEFORM
    return BrickGrid((n, n, n), index, values, dfm, background=1.0)


def run_band(device, n=2048, steps=10, warmup=3, dense_n=512):
    """Narrow-band extraction.  (1) The benchmark's spheres as a band at n^3 (built
    without a dense grid, sphere_band), DiffDMC forward + backward with quads and deform:
    its dense grids (SDF, deform and their gradients, 32 B per point) would not fit in
    HBM at 2048^3.  (2) The headline's own grid at dense_n^3 cut to a band
    (BrickGrid.from_dense: every brick with an end of a crossing edge), the same step on
    the band and on the dense grid (recompute backward): the same mesh, and the time of
    each."""
    from diso_gb300 import BrickGrid, DiffDMC

    def step_fn(mod, band):
        v, q = mod.forward_bricks(band, return_quads=True)
        w = loss_weights(v.shape[0], device, v.dtype)
        (v * w).sum().backward()
        return v, q

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, out

    out = {}
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    band = sphere_band(n, device)
    band.values.requires_grad_(True)
    band.deform.requires_grad_(True)
    mod = DiffDMC(torch.float32)
    band_bytes = sum(t.numel() * t.element_size() for t in (band.index, band.values, band.deform))
    torch.cuda.reset_peak_memory_stats(device)

    def big():
        band.values.grad = None
        band.deform.grad = None
        return step_fn(mod, band)

    ms, (v, q) = timed(big)
    # per-kernel times of the same step (CUDA events around every launch)
    mod._ex.timing(True)
    for _ in range(steps):
        big()
    torch.cuda.synchronize()
    kern = {k: round(t / steps, 4) for k, (c, t) in mod._ex.timing_read().items()}
    mod._ex.timing(False)
    out["band"] = {"n": n, "bricks": band.count, "verts": v.shape[0], "quads": q.shape[0], "ms_per_step": ms,
                   "kernel_ms_per_step": kern,
                   "grids_s": 1e3 / ms, "band_gb": round(band_bytes / 1e9, 3),
                   "peak_hbm_gb": round(torch.cuda.max_memory_allocated(device) / 1e9, 3),
                   "extractor_scratch_gb": round(mod._ex.scratch_bytes() / 1e9, 3),
                   "dense_equivalent_gb": round(n ** 3 * 4 * (1 + 3) * 2 / 1e9, 1)}
    del band, v, q, mod
    torch.cuda.empty_cache()
    # the headline grid as a band
    sdf = spheres_field(dense_n, device)
    dfm = deform_field(dense_n, device)
    cut = BrickGrid.from_dense(sdf, 0.0, deform=dfm)
    cut.values.requires_grad_(True)
    cut.deform.requires_grad_(True)
    mod = DiffDMC(torch.float32, recompute=True)
    s_req, d_req = sdf.clone().requires_grad_(True), dfm.clone().requires_grad_(True)

    def dense_step():
        s_req.grad = None
        d_req.grad = None
        v, q = mod(s_req, d_req, return_quads=True)
        (v * loss_weights(v.shape[0], device, v.dtype)).sum().backward()
        return v, q

    def band_step():
        cut.values.grad = None
        cut.deform.grad = None
        return step_fn(mod, cut)

    ms_d, (vd, qd) = timed(dense_step)
    ms_b, (vb, qb) = timed(band_step)
    out["headline_grid_as_band"] = {"n": dense_n, "bricks": cut.count,
                                    "bricks_share": round(cut.count / ((dense_n + 7) // 8) ** 3, 4),
                                    "same_mesh": bool(torch.equal(vd, vb) and torch.equal(qd, qb)),
                                    "dense_ms": ms_d, "band_ms": ms_b}
    return out


def run_configs(device, steps=5, warmup=2):
    """The reference's other published configurations, device-resident, forward +
    backward (loss = sum(verts * w), w ~ N(0, 1) seeded; the first configuration sums
    the vertices): the 64^3 sphere (MC, fp32, no deform) and the 256^3 round cube and
    U(-1, 1) random init (MC, DMC quads and DMC triangles; fp32 and fp64; deform
    U(-0.45, 0.45)).  ms per step; the same fields as tests/test_gpu_config256.py."""
    from diso_gb300 import DiffDMC, DiffMC

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps

    out = {}
    a = torch.linspace(-1, 1, 64, device=device)
    sphere = torch.sqrt(a.view(-1, 1, 1) ** 2 + a.view(1, -1, 1) ** 2 + a.view(1, 1, -1) ** 2) - 0.5
    s1 = sphere.clone().requires_grad_(True)
    mc = DiffMC(torch.float32)

    def first():
        s1.grad = None
        v, _ = mc(s1)
        v.sum().backward()

    out["sphere64_mc_f32"] = round(timed(first), 4)
    n = 256
    g = torch.Generator(device=device).manual_seed(0)
    a = torch.linspace(-1, 1, n, device=device, dtype=torch.float64)
    X, Y, Z = a.view(-1, 1, 1), a.view(1, -1, 1), a.view(1, 1, -1)
    q = [torch.clamp(c.abs() - 0.5, min=0) for c in (X, Y, Z)]
    fields = {"roundcube": torch.sqrt(q[0] ** 2 + q[1] ** 2 + q[2] ** 2) - 0.1,
              "random": torch.rand((n, n, n), device=device, dtype=torch.float64, generator=g) * 2 - 1}
    dfm64 = (torch.rand((n, n, n, 3), device=device, dtype=torch.float64, generator=g) - 0.5) * 0.9
    for name, f64 in fields.items():
        for dt in (torch.float32, torch.float64):
            sdf, dfm = f64.to(dt).contiguous(), dfm64.to(dt)
            for method, rq in (("mc", None), ("dmc_quads", True), ("dmc_tris", False)):
                mod = DiffMC(dt) if method == "mc" else DiffDMC(dt)
                kw = {} if rq is None else {"return_quads": rq}
                s = sdf.clone().requires_grad_(True)
                d = dfm.clone().requires_grad_(True)
                v, _ = mod(s, d, **kw)
                w = torch.randn(v.shape, dtype=dt, device=device, generator=torch.Generator(device).manual_seed(1))
                del v

                def step():
                    s.grad = None
                    d.grad = None
                    vv, _ = mod(s, d, **kw)
                    (vv * w).sum().backward()

                out[f"{name}{n}_{method}_{str(dt)[-7:]}"] = round(timed(step), 4)
                del s, d, w
            del sdf, dfm
    return {"ms_per_step": out, "note": "device-resident inputs; 64^3: loss = sum(verts); 256^3: deform, "
                                        "loss = sum(verts * w)"}


def octahedron_mlp(device, width=64, seed=SEED):
    """A ReLU MLP SDF: |x| + |y| + |z| - 0.8 (|t| = relu(t) + relu(-t)) plus a seeded
    random ReLU branch of `width` units scaled by 0.05."""
    from torch import nn

    g = torch.Generator().manual_seed(seed)
    net = nn.Sequential(nn.Linear(3, 6 + width), nn.ReLU(), nn.Linear(6 + width, 1 + width), nn.ReLU(),
                        nn.Linear(1 + width, 1))
    with torch.no_grad():
        for m in net:
            if isinstance(m, nn.Linear):
                m.weight.zero_()
                m.bias.zero_()
        net[0].weight[:3] = torch.eye(3)
        net[0].weight[3:6] = -torch.eye(3)
        net[0].weight[6:] = torch.randn((width, 3), generator=g) * 0.7
        net[0].bias[6:] = torch.randn(width, generator=g) * 0.2
        net[2].weight[0, :6] = 1.0
        net[2].weight[1:, 6:] = torch.randn((width, width), generator=g) * (0.3 * (32 / width) ** 0.5)
        net[4].weight[0, 0] = 1.0
        net[4].weight[0, 1:] = torch.randn(width, generator=g) * 0.05
        net[4].bias.fill_(-0.8)
    return net.to(device)


def run_mlp(device, n=256, steps=5, warmup=2):
    """An MLP SDF (octahedron_mlp, fp32) on an n^3 grid, DiffDMC quads, forward +
    backward to the network's parameters: from its narrow band (MLPField: interval
    bounds per brick, the network evaluated at the band's points only) against the
    network evaluated on the whole grid and the dense path.  The same mesh (up to the
    rounding of evaluating a point inside one batch or another).  The dense path keeps
    the network's activations at every grid point for its backward (about 1 KB per
    point), hence the moderate default size."""
    from diso_gb300 import DiffDMC, MLPField

    net = octahedron_mlp(device)
    field = MLPField(net)
    mod = DiffDMC(torch.float32)

    def band_step():
        net.zero_grad(set_to_none=True)
        v, q = mod.forward_mlp(field, (n, n, n), return_quads=True)
        (v * loss_weights(v.shape[0], device, v.dtype)).sum().backward()
        return v, q

    def dense_step():
        net.zero_grad(set_to_none=True)
        v, q = mod(field.dense((n, n, n)), return_quads=True)
        (v * loss_weights(v.shape[0], device, v.dtype)).sum().backward()
        return v, q

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            out = fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / steps, out

    ms_b, (vb, qb) = timed(band_step)
    ms_d, (vd, qd) = timed(dense_step)
    band = field.band((n, n, n), 0.0)
    return {"field": f"ReLU MLP 3-70-65-1 (octahedron + random branch) at {n}^3, DiffDMC quads, fwd+bwd to the weights",
            "bricks": band.count, "bricks_share": round(band.count / band.index.numel(), 4),
            "verts": vb.shape[0], "same_faces": bool(torch.equal(qb, qd)),
            "max_vertex_diff": float((vb - vd).detach().abs().max()) if vb.shape == vd.shape else None,
            "dense_ms": ms_d, "band_ms": ms_b, "speedup": ms_d / ms_b}


def run_served(device, nreq=20000, rate=2000.0, plain_sample=4000):
    """The served stream: p50 / p99 latency and grids/s of the continuous-batching
    server on the Poisson trace in real time, and its capacity (the whole trace
    available at once) against the plain per-request call's capacity on the same
    requests (a prefix of `plain_sample` of them: the trace is i.i.d.).  In real
    time the server's grids/s cannot exceed the arrival rate, so the speedup is the
    ratio of capacities."""
    from diso_gb300.serve import Server, serve_plain, summarize

    pool = InputPool(device)
    pool.warm()
    srv = Server(device, hbm_budget=60e9, max_batch=64, workers=4)
    srv.serve(served_trace(128, rate, seed=11, pool=pool), realtime=False)  # warm-up
    trace = served_trace(nreq, rate, pool=pool)
    srv.serve(trace)
    realtime = summarize(trace)
    peak = srv.peak
    cap_trace = served_trace(nreq, rate, pool=pool)
    srv.serve(cap_trace, realtime=False)
    capacity = {k: v for k, v in summarize(cap_trace, t_first=0.0).items() if not k.startswith("p")}
    srv.close()
    serve_plain(served_trace(64, rate, seed=11, pool=pool), device, realtime=False)  # warm-up
    plain_trace = served_trace(nreq, rate, pool=pool)[:plain_sample]
    serve_plain(plain_trace, device, realtime=False)
    plain = {k: v for k, v in summarize(plain_trace, t_first=0.0).items() if not k.startswith("p")}
    bound, per = device_bound(trace, pool, device)
    heavy = sorted(per.items(), key=lambda kv: -kv[1])[:3]
    return {"requests": nreq, "rate_per_s": rate, "server_realtime": realtime, "server_capacity": capacity,
            "plain_per_request_capacity": plain, "plain_sample": plain_sample,
            "plain_kernel_bound_grids_s": bound,
            "plain_kernel_ms_heaviest": {f"{n}^3 {k} {'mc' if m == 0 else 'dmc'}": round(v, 3) for (n, k, m), v in heavy},
            "grids_s_speedup": capacity["grids_per_s"] / plain["grids_per_s"], "peak_budget_gb": peak / 1e9,
            "inputs": "device-resident pool: 4 grids per (N, kind), one N(0,1) gradient buffer",
            "workers": 4, "max_batch": 64}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "100",
                 "-i", str(self.gpu)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx = float(p[2])
            except ValueError:
                continue
            for name, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def smi_id(device):
    """nvidia-smi -i argument of a torch device: its PCI bus id when torch exposes it."""
    p = torch.cuda.get_device_properties(device)
    if hasattr(p, "pci_bus_id") and hasattr(p, "pci_domain_id") and hasattr(p, "pci_device_id"):
        return f"{p.pci_domain_id:08x}:{p.pci_bus_id:02x}:{p.pci_device_id:02x}.0"
    return str(device.index or 0)


# ----------------------------------------------------------------------------- ours
class PhaseEvents:
    def __init__(self):
        self.open = {}
        self.done = {}

    def __call__(self, name, what):
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        if what == "start":
            self.open[name] = ev
        else:
            self.done.setdefault(name, []).append((self.open.pop(name), ev))

    def mean_ms(self):
        return {k: sum(a.elapsed_time(b) for a, b in v) / len(v) for k, v in self.done.items()}


def kernel_bytes(vol, nseg, nv, nq, s, zshare, active_pts, zeros_in_fused=True):
    """Algorithmic bytes per launch of each kernel of the 512^3 DMC step: what the
    kernel's function must read and write at least (nq crossing edges = quads, nv
    patches = vertices, s bytes per scalar, active_pts = points of the point tiles
    with a crossing edge nearby).

    Stored mode: the forward's count and emit also write the zeros of the two
    gradient arrays (the count the share zshare, the emit the rest; memsets,
    "zero_grads", when the buffers do not allow it) and the emit the edge record;
    the backward's edge pass and gather read it.  Recompute mode: the forward writes
    no zeros and no record; the backward zeroes the point tiles with no crossing
    nearby and recomputes the rest in one pass (fused_bwd); the zeros are bulk copies
    issued by the fused pass itself (zeros_in_fused) or, for grids whose rows are no
    multiple of 16 bytes, a kernel of their own (zero_tiles)."""
    zeros = vol * 4 * s
    return {
        # the SDF once; the per-segment counts out; its share of the zeros (stored mode)
        "count": vol * s + nseg * 8 + zshare * zeros,
        # segment counts in and out
        "scan": 2 * nseg * 8,
        # both end points of every crossing edge (SDF + deform) in; vertices and quads out;
        # stored mode: the edge record (cell + axis, four patch ids, a byte per vertex) and
        # the rest of the zeros
        "emit": 2 * nq * 4 * s + nv * 3 * s + nq * 4 * 8 + (nq * (8 + 16) + nv + (1 - zshare) * zeros if zshare else 0),
        "zero_grads": zeros,
        # per edge: record (cell, 4 patch ids), 4 patch bytes and 4 dL/dverts in, end points
        # (SDF + deform) in, 2 x 4 adjoints out
        "edge": nq * (8 + 16 + 4 + 4 * 3 * s + 2 * 4 * s + 8 * s),
        # the adjoints of every edge, once from each end
        "gather": nq * 8 * s,
        # the gradients of the point tiles with no crossing nearby
        "zero_tiles": (vol - active_pts) * 4 * s,
        # the SDF of the active tiles in, their gradients out; the deform at both ends of
        # every crossing edge and dL/dverts in; the other tiles' zeros when it writes them
        "fused_bwd": active_pts * 5 * s + nq * 2 * 3 * s + nv * 3 * s
        + ((vol - active_pts) * 4 * s if zeros_in_fused else 0),
    }


def active_points(sdf, iso=0.0):
    """Points of the 4 x 8 x 32 point tiles that hold a point with a crossing edge
    (the tiles the backward's fused pass works on; the grid is padded with
    iso + 1 as in the forward)."""
    with torch.no_grad():
        b = torch.nn.functional.pad(sdf.unsqueeze(0).unsqueeze(0) >= iso, (1, 1, 1, 1, 1, 1), value=True)[0, 0]
        inc = torch.zeros_like(b, dtype=torch.bool)
        for ax in range(3):
            c = b.narrow(ax, 1, b.shape[ax] - 1) != b.narrow(ax, 0, b.shape[ax] - 1)
            inc.narrow(ax, 1, b.shape[ax] - 1).logical_or_(c)
            inc.narrow(ax, 0, b.shape[ax] - 1).logical_or_(c)
        inner = inc[1:-1, 1:-1, 1:-1]
        n0, n1, n2 = inner.shape
        t = torch.zeros(((n0 + 3) // 4) * 4, ((n1 + 7) // 8) * 8, ((n2 + 31) // 32) * 32, dtype=torch.bool,
                        device=sdf.device)
        t[:n0, :n1, :n2] = inner
        act = t.view(t.shape[0] // 4, 4, t.shape[1] // 8, 8, t.shape[2] // 32, 32).any(5).any(3).any(1)
        return int(act.sum()) * 4 * 8 * 32


def read_profile_traffic(kernel, n):
    """Per-launch DRAM bytes of `kernel` on the n^3 workload from the committed ncu
    summary of that size (profiles/dram_traffic_*_<n>.txt, lines "<kernel>: <bytes>"),
    None when there is none."""
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", f"dram_traffic_*_{n}.txt"))):
        try:
            txt = open(path).read()
        except OSError:
            continue
        m = re.search(r"^%s:\s*([0-9.eE+]+)\s*$" % re.escape(kernel), txt, flags=re.M)
        if m:
            return float(m.group(1))
    return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def max_over_ranks(ms, world, device):
    """The slowest rank's time: every rank's `ms` reduced with MAX over the job's
    ranks (replicas: the job ends when its last rank does); no collective for one."""
    t = torch.tensor([ms], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, steps, ms):
    """Grids per second of the whole job: each of the `world` replicas runs `steps`
    grids (weak scaling) within `ms`, the slowest rank's time."""
    return world * steps / (ms / 1e3)


def time_steps(ext, s, d, w, steps, warmup, world, with_clocks=False):
    """`steps` timed forward + backward steps of `ext` on the resident inputs (after
    `warmup` untimed ones), bracketed by barrier + synchronize, with CUDA events on
    the stream around the whole loop only; then the same number of steps again with
    CUDA events around every launch of the extractor (its timing mode) and around
    the phases, for the per-kernel breakdown.  Returns (ms over the first loop's
    steps, max over ranks; per-kernel totals and phase means of the second loop;
    clocks sampled during the first)."""
    import diso_gb300.extraction as X

    def step():
        s.grad = None
        d.grad = None
        v, _ = ext(s, d, return_quads=True)
        (v * w).sum().backward()

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clk = ClockSampler(smi_id(s.device)) if with_clocks else None
    if clk:
        clk.__enter__()
    try:
        t0.record()
        for _ in range(steps):
            step()
        t1.record()
        torch.cuda.synchronize()
    finally:
        if clk:
            clk.__exit__()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms = max_over_ranks(t0.elapsed_time(t1), world, s.device)
    ph = PhaseEvents()
    X.phase_timer = ph
    ext._ex.timing(True)  # CUDA events around every launch of the extractor, on its stream
    try:
        for _ in range(steps):
            step()
        torch.cuda.synchronize()
    finally:
        X.phase_timer = None
    kernels = ext._ex.timing_read()
    ext._ex.timing(False)
    return ms, kernels, ph.mean_ms(), (clk.summary() if clk else None)


def peak_memory(ext, s, d, w):
    """Device memory of one forward + backward step: the peak of torch's allocator
    over the step (inputs, outputs, gradients, per-call records) plus the
    extractor's own scratch, and what the forward keeps alive until its backward
    beyond the inputs and the returned mesh."""
    s.grad = None
    d.grad = None
    torch.cuda.synchronize()
    base = torch.cuda.memory_allocated(s.device)
    torch.cuda.reset_peak_memory_stats(s.device)
    v, f = ext(s, d, return_quads=True)
    loss = (v * w).sum()
    torch.cuda.synchronize()
    held = torch.cuda.memory_allocated(s.device) - base - v.numel() * v.element_size() - f.numel() * f.element_size()
    loss.backward()
    torch.cuda.synchronize()
    peak = torch.cuda.max_memory_allocated(s.device) + ext._ex.scratch_bytes()
    del v, f, loss
    return {"peak_hbm_gb": round(peak / 1e9, 4), "held_fwd_to_bwd_gb": round(max(held, 0) / 1e9, 4),
            "extractor_scratch_gb": round(ext._ex.scratch_bytes() / 1e9, 4)}


def run_ours(args, rank, world, device):
    from diso_gb300 import DiffDMC, tune
    from diso_gb300 import _native as N

    n = args.n
    sdf = spheres_field(n, device)
    deform = deform_field(n, device)
    # the large configuration: the backward recomputes the crossing lists
    ext = DiffDMC(torch.float32, recompute=True)
    # launch widths from the package's autotuner (timed on a synthetic field of this
    # size, outside the timed region; cached per GPU, method, dtype, size and mode)
    tuned = (tune.tune_module(ext, (n, n, n), retune=args.retune) if not args.no_tune else
             {"params": {}, "ms": 0.0, "default_ms": 0.0, "trials": 0})
    s = sdf.clone().requires_grad_(True)
    d = deform.clone().requires_grad_(True)
    v, f = ext(s, d, return_quads=True)
    nv, nq = v.shape[0], f.shape[0]
    w = loss_weights(nv, device, torch.float32)
    del v, f

    ms_max, kernels, phases, clocks = time_steps(ext, s, d, w, args.steps, args.warmup, world, with_clocks=True)
    mem = peak_memory(ext, s, d, w)

    # the same workload with the forward's edge record and gradient buffers kept for
    # the backward (stored mode), for comparison
    stored = DiffDMC(torch.float32, recompute=False)
    tuned_st = tune.tune_module(stored, (n, n, n), retune=args.retune) if not args.no_tune else {"params": {}}
    ms_st, k_st, ph_st, _ = time_steps(stored, s, d, w, args.steps, args.warmup, world)
    mem_st = peak_memory(stored, s, d, w)
    del stored

    # e2e: every step's inputs are copied from pinned host memory, and its mesh
    # (verts, quads), both gradients and the loss are copied back into pinned host
    # memory.  Inputs are double-buffered (step k+1's copy runs on a copy stream while
    # step k computes), results go back on a third stream while the next step
    # computes; every copy lies inside the timed region.
    e2e_steps = max(3, min(args.steps, args.e2e_steps))
    sdf_h = sdf.cpu().pin_memory()
    def_h = deform.cpu().pin_memory()
    bufs = [(torch.empty_like(sdf), torch.empty_like(deform)) for _ in range(2)]
    out_h = [{"verts": torch.empty((nv, 3), dtype=torch.float32, pin_memory=True),
              "quads": torch.empty((nq, 4), dtype=torch.int64, pin_memory=True),
              "grad_sdf": torch.empty(sdf.shape, dtype=torch.float32, pin_memory=True),
              "grad_deform": torch.empty(deform.shape, dtype=torch.float32, pin_memory=True)} for _ in range(2)]
    copy_stream = torch.cuda.Stream(device)
    back_stream = torch.cuda.Stream(device)
    ready = [torch.cuda.Event(), torch.cuda.Event()]
    done = [torch.cuda.Event(), torch.cuda.Event()]  # the compute that read buffer i has finished
    back_done = [torch.cuda.Event(), torch.cuda.Event()]  # host buffers i are free again
    d2h = {"bytes": 0}

    def issue_copy(i):
        copy_stream.wait_event(done[i])
        with torch.cuda.stream(copy_stream), torch.no_grad():
            bufs[i][0].copy_(sdf_h, non_blocking=True)
            bufs[i][1].copy_(def_h, non_blocking=True)
            ready[i].record(copy_stream)

    def issue_back(i, tensors, cur):
        back_stream.wait_event(back_done[i])
        back_stream.wait_stream(cur)
        nbytes = 0
        with torch.cuda.stream(back_stream):
            for name, t in tensors.items():
                dst = out_h[i][name]
                if dst.shape != t.shape:
                    dst = out_h[i][name] = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
                dst.copy_(t, non_blocking=True)
                t.record_stream(back_stream)
                nbytes += t.numel() * t.element_size()
            back_done[i].record(back_stream)
        d2h["bytes"] = nbytes

    def e2e_run(k_steps):
        cur = torch.cuda.current_stream(device)
        copy_stream.wait_stream(cur)
        issue_copy(0)
        for k in range(k_steps):
            i = k % 2
            if k + 1 < k_steps:
                issue_copy(1 - i)
            cur.wait_event(ready[i])
            sg = bufs[i][0].requires_grad_(True)
            dg = bufs[i][1].requires_grad_(True)
            sg.grad = None
            dg.grad = None
            v, q = ext(sg, dg, return_quads=True)
            loss = (v * w).sum()
            loss.backward()
            issue_back(i, {"verts": v.detach(), "quads": q, "grad_sdf": sg.grad, "grad_deform": dg.grad}, cur)
            loss.item()
            done[i].record(cur)
        back_stream.synchronize()

    e2e_run(2)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    e2e_run(e2e_steps)
    e1.record()
    torch.cuda.synchronize()
    e_ms = max_over_ranks(e0.elapsed_time(e1), world, device)

    # roofline of the dominant kernel (per-launch event times of the timed region)
    s_b = 4
    vol = n ** 3
    nseg = (n + 1) ** 2 * ((n + 1 + 31) // 32)
    act_pts = active_points(sdf)
    algo = kernel_bytes(vol, nseg, nv, nq, s_b, 0.0, act_pts, zeros_in_fused="zero_tiles" not in kernels)
    zshare = 0.0 if "zero_grads" in k_st else float(N.lib().diso_zero_count_share())
    algo_st = kernel_bytes(vol, nseg, nv, nq, s_b, zshare, act_pts)
    per_launch = {k: ms / max(cnt, 1) for k, (cnt, ms) in kernels.items()}
    ours = {k: v for k, v in per_launch.items() if k in algo and k != "zero_grads"}
    dom = max(ours, key=lambda k: ours[k] * kernels[k][0])
    peak, peak_kind = measured_peaks()
    achieved = algo[dom] / (per_launch[dom] * 1e-3) / 1e9
    traffic = read_profile_traffic(dom, n)
    step_bytes = vol * s_b * (3 + 3) + 4 * nq * 3 * s_b + 2 * nv * 3 * s_b + 8 * nq * 4
    ms_step = ms_max / args.steps
    res = {
        "metric": metric_name(n),
        "value": job_throughput(world, args.steps, ms_max),
        "unit": "grids/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": f"synthetic: min of 16 seeded spheres + 0.01*N(0,1) noise at {n}^3, deform U(-0.45,0.45)",
        "config": {"workload": f"dmc_fwd_bwd_{n}_spheres16", "n": n, "method": "DiffDMC", "return_quads": True,
                   "deform": True, "normalize": True, "backward": "recompute", "verts": nv, "quads": nq,
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}",
                   "phase_ms": {k: round(v, 4) for k, v in phases.items()},
                   "kernel_ms_per_step": {k: round(ms / args.steps, 4) for k, (cnt, ms) in kernels.items()},
                   "kernel_gbs": {k: round(algo[k] / (per_launch[k] * 1e-3) / 1e9, 1) for k in per_launch
                                  if k in algo},
                   "active_point_tiles": act_pts // 1024,
                   "launch": {"tuned": tuned["params"], "tuned_ms": round(tuned["ms"], 4),
                              "default_ms": round(tuned["default_ms"], 4), "trials": tuned["trials"]},
                   "step_algorithmic_gb": round(step_bytes / 1e9, 4),
                   "step_algorithmic_gbs": step_bytes / (ms_step * 1e-3) / 1e9,
                   "step_hbm_frac": step_bytes / (ms_step * 1e-3) / 1e9 / peak},
        "peak_hbm_gb": mem["peak_hbm_gb"],
        "memory": mem,
        "stored_mode": {"backward": "stored edge record", "ms_per_step": ms_st / args.steps,
                        "launch": tuned_st["params"],
                        "kernel_gbs": {k: round(algo_st[k] / (ms / max(cnt, 1) * 1e-3) / 1e9, 1)
                                       for k, (cnt, ms) in k_st.items() if k in algo_st},
                        "grids_s": job_throughput(world, args.steps, ms_st),
                        "step_hbm_frac": step_bytes / (ms_st / args.steps * 1e-3) / 1e9 / peak,
                        "kernel_ms_per_step": {k: round(ms / args.steps, 4) for k, (cnt, ms) in k_st.items()},
                        **mem_st},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes": algo[dom],
                     "ms_per_launch": per_launch[dom], "traffic": traffic},
        "e2e": {"value": job_throughput(world, e2e_steps, e_ms), "unit": "grids/s",
                "h2d_bytes_per_step": int(sdf.numel() * 4 + deform.numel() * 4),
                "d2h_bytes_per_step": int(d2h["bytes"]) + 4,
                "d2h": "verts, quads, grad_sdf, grad_deform and the loss"},
        # the timed kernels, and the count_prep_kernel launched before every count
        "gpu_launches": sum(cnt for k, (cnt, _) in kernels.items() if k != "zero_grads")
        + kernels.get("count", (0, 0.0))[0],
        "clocks": clocks,
    }
    return res


# ----------------------------------------------------------------------------- reference CUDA
def run_reference_cuda(args, device):
    """The reference's own DiffDMC forward + backward on the same field, through its
    unmodified Python API over its CUDA extension, built from a reference checkout
    named by the environment variable DISO_REFERENCE_SRC (the recipe in oracle/ builds
    it into oracle/_ref/).  Without a checkout on this machine the entry says so."""
    src = os.environ.get("DISO_REFERENCE_SRC")
    if not src or not os.path.exists(os.path.join(src, "src", "cudualmc.cu")):
        return {"unavailable": "no reference checkout on this machine (set DISO_REFERENCE_SRC to one to time "
                               "the reference's CUDA path here)"}
    try:
        from oracle.build_ref import load_reference

        ref = load_reference(src)
        n = args.n
        s = spheres_field(n, device).requires_grad_(True)
        d = deform_field(n, device).requires_grad_(True)
        ext = ref.DiffDMC(dtype=torch.float32)
        v, _ = ext(s, d, return_quads=True)
        w = loss_weights(v.shape[0], device, torch.float32)

        def step():
            s.grad = None
            d.grad = None
            v, _ = ext(s, d, return_quads=True)
            (v * w).sum().backward()

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(args.steps):
            step()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / args.steps
        return {"ms_per_step": ms, "grids_s": 1e3 / ms, "steps": args.steps, "warmup": args.warmup,
                "source": "reference DiffDMC (its own Python API and CUDA extension, built for sm_103a)"}
    except Exception as e:  # report, but keep the headline line
        return {"unavailable": f"reference build or run failed: {repr(e)[:200]}"}


# ----------------------------------------------------------------------------- CPU
def cpu_sample(n, sdf, deform, w, planes):
    """Oracle fwd+bwd on a slab of `planes` x-planes from the middle of the grid; returns seconds."""
    from oracle import oracle as O

    lo = max(0, n // 2 - planes // 2)
    s = sdf[lo:lo + planes]
    d = deform[lo:lo + planes]
    t = time.perf_counter()
    v, q, _ = O.extract(O.DMC, s, d, 0.0, True, True, "float32")
    ww = np.resize(w, v.shape)
    O.backward(O.DMC, s, d, ww, 0.0, True, "float32")
    return time.perf_counter() - t


def run_cpu(args, steps, warmup, budget_s):
    from oracle import oracle as O

    n = args.n
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    sdf = spheres_field(n, dev).double().cpu().numpy()
    deform = deform_field(n, dev).double().cpu().numpy()
    w = np.random.default_rng(SEED + 200).standard_normal((1 << 16, 3))
    # size the sample: time a thin slab, then scale to ~budget_s per step (at most the whole grid)
    probe = max(8, n // 32)
    t = cpu_sample(n, sdf, deform, w, probe)
    planes = int(min(n, max(probe, probe * budget_s / max(t, 1e-3))))
    times = []
    for i in range(warmup + steps):
        dt = cpu_sample(n, sdf, deform, w, planes)
        if i >= warmup:
            times.append(dt)
    frac = planes / n
    value = frac / statistics.mean(times)
    return value, planes, O.num_threads(), statistics.mean(times)


# ----------------------------------------------------------------------------- main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU work per baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--retune", action="store_true", help="time the launch widths again instead of the cached ones")
    ap.add_argument("--no-tune", action="store_true", help="the library's default launch widths (for profiling)")
    ap.add_argument("--no-batched", action="store_true", help="skip the uneven-batch and served measurements")
    ap.add_argument("--requests", type=int, default=20000, help="served-trace length")
    ap.add_argument("--band-n", type=int, default=2048, help="grid size of the narrow-band measurement")
    ap.add_argument("--only", choices=["narrow_band", "fused_field", "mesh_consumers", "mlp_field", "configs"],
                    help="run one side measurement alone and print it (for profiling)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        steps, warmup = args.steps, args.warmup
        # each step a bounded sample, sized so that the whole run stays within ~3 minutes
        budget = min(20.0, max(0.1, 180.0 / max(1, steps + warmup)))
        value, planes, cores, sec = run_cpu(args, steps, warmup, budget_s=budget)
        out = {"metric": metric_name(args.n), "value": value, "unit": "grids/s", "n_gpus": args.gpus, "steps": steps,
               "warmup": warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic (same field as ours)",
               "config": {"workload": f"dmc_fwd_bwd_{args.n}_spheres16", "n": args.n, "method": "DiffDMC",
                          "return_quads": True, "deform": True, "normalize": True,
                          "sample": f"middle {planes} of {args.n} x-planes per step"},
               "impl": "reference",
               "cpu_baseline": {"value": value, "unit": "grids/s", "cores": cores, "kind": "port",
                                "sample": f"OpenMP FP64 oracle, middle {planes}/{args.n} x-planes, "
                                          f"scaled by the volume fraction"},
               "e2e": {"value": value, "unit": "grids/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out), flush=True)
        return

    if args.only:
        device = torch.device("cuda", torch.cuda.current_device())
        fn = {"narrow_band": lambda: run_band(device, args.band_n, steps=args.steps, warmup=args.warmup),
              "fused_field": lambda: run_field(device, args.n, steps=args.steps, warmup=args.warmup),
              "mesh_consumers": lambda: run_mesh(device, args.n, steps=args.steps, warmup=args.warmup),
              "mlp_field": lambda: run_mlp(device, args.n, steps=args.steps, warmup=args.warmup),
              "configs": lambda: run_configs(device, steps=args.steps, warmup=args.warmup)}[args.only]
        print(json.dumps({args.only: fn()}), flush=True)
        return
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    device = torch.device("cuda", torch.cuda.current_device())
    res = run_ours(args, rank, world, device)
    if rank == 0:
        res["reference_cuda"] = run_reference_cuda(args, device)
    if rank == 0 and world == 1 and not args.no_batched:
        for name, fn in (("batched_mc", lambda: run_batched(device, 0)), ("batched_dmc", lambda: run_batched(device, 1)),
                         ("served", lambda: run_served(device, args.requests)),
                         ("mesh_consumers", lambda: run_mesh(device, args.n)),
                         ("fused_field", lambda: run_field(device, args.n)),
                         ("narrow_band", lambda: run_band(device, args.band_n)),
                         ("mlp_field", lambda: run_mlp(device, 256)),
                         ("configs", lambda: run_configs(device))):
            try:
                res[name] = fn()
            except Exception as e:  # report, but keep the headline line
                res[name] = {"error": repr(e)[:300]}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        value, planes, cores, sec = run_cpu(args, 1, 0, args.cpu_budget)
        res["cpu_baseline"] = {"value": value, "unit": "grids/s", "cores": cores, "kind": "port",
                               "sample": f"OpenMP FP64 oracle on the middle {planes}/{args.n} x-planes, "
                                         f"{sec:.1f} s, scaled by the volume fraction"}
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
