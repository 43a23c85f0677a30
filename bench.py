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
memory each step and the loss read back.  ``--impl reference`` times the CPU
implementation of the same path (the reference has no CPU code; the project's
OpenMP FP64 restatement in oracle/ stands in) on bounded samples of the grid.
Under torchrun each rank runs its own replica of the workload (no collective on
the data path); the time is the max over ranks.
"""
from __future__ import annotations

import argparse
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
METRIC = "fwd+bwd grids/s @512^3 (DiffDMC, fp32, deform, return_quads)"
PROFILE = os.path.join(ROOT, "profiles", "dmc_backward_512.txt")


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


def read_profile_traffic():
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    try:
        txt = open(PROFILE).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_ours(args, rank, world, device):
    from diso_gb300 import DiffDMC
    import diso_gb300.extraction as X

    n = args.n
    sdf = spheres_field(n, device)
    deform = deform_field(n, device)
    ext = DiffDMC(torch.float32)
    s = sdf.clone().requires_grad_(True)
    d = deform.clone().requires_grad_(True)
    v, f = ext(s, d, return_quads=True)
    nv, nq = v.shape[0], f.shape[0]
    w = loss_weights(nv, device, torch.float32)
    del v, f

    def step(s_in, d_in):
        s_in.grad = None
        d_in.grad = None
        v, _ = ext(s_in, d_in, return_quads=True)
        (v * w).sum().backward()

    for _ in range(args.warmup):
        step(s, d)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ph = PhaseEvents()
    X.phase_timer = ph
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(smi_id(device)) as clk:
        t0.record()
        for _ in range(args.steps):
            step(s, d)
        t1.record()
        torch.cuda.synchronize()
    X.phase_timer = None
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ms = t0.elapsed_time(t1)
    ms_t = torch.tensor([ms], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(ms_t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(ms_t.item())
    phases = ph.mean_ms()

    # e2e: inputs from pinned host memory every step, loss read back
    e2e_steps = max(3, min(args.steps, args.e2e_steps))
    sdf_h = sdf.cpu().pin_memory()
    def_h = deform.cpu().pin_memory()
    s2 = torch.empty_like(sdf)
    d2 = torch.empty_like(deform)

    def e2e_step():
        with torch.no_grad():
            s2.copy_(sdf_h, non_blocking=True)
            d2.copy_(def_h, non_blocking=True)
        sg = s2.requires_grad_(True)
        dg = d2.requires_grad_(True)
        sg.grad = None
        dg.grad = None
        v, _ = ext(sg, dg, return_quads=True)
        loss = (v * w).sum()
        loss.backward()
        return loss.item()

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(e2e_steps):
        e2e_step()
    e1.record()
    torch.cuda.synchronize()
    e_ms = torch.tensor([e0.elapsed_time(e1)], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(e_ms, op=torch.distributed.ReduceOp.MAX)
    e_ms = float(e_ms.item())

    # roofline of the dominant phase
    s_b = 4
    vol = n ** 3
    algo = {
        # SDF read (the dense pass); the per-segment counts and their scan are design overhead
        "count": vol * s_b,
        # deform gathers at both ends of every crossing, SDF of the active tiles, vertices and quads out
        "emit": 2 * nq * 3 * s_b + nv * 3 * s_b + nq * 4 * 8,
        # SDF re-read, dL/dsdf and dL/ddeform written, dL/dverts read, deform gathered at crossings
        "backward": vol * s_b * (1 + 1 + 3) + nv * 3 * s_b + 2 * nq * 3 * s_b,
    }
    dom = max((k for k in phases if k in algo), key=lambda k: phases[k])
    peak, peak_kind = measured_peaks()
    achieved = algo[dom] / (phases[dom] * 1e-3) / 1e9
    traffic = read_profile_traffic() if dom == "backward" else None
    step_bytes = vol * s_b * (3 + 3) + 4 * nq * 3 * s_b + 2 * nv * 3 * s_b + 8 * nq * 4
    ms_step = ms_max / args.steps
    res = {
        "metric": METRIC,
        "value": world * args.steps / (ms_max / 1e3),
        "unit": "grids/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: min of 16 seeded spheres + 0.01*N(0,1) noise at 512^3, deform U(-0.45,0.45)",
        "config": {"workload": f"dmc_fwd_bwd_{n}_spheres16", "n": n, "method": "DiffDMC", "return_quads": True,
                   "deform": True, "normalize": True, "verts": nv, "quads": nq,
                   "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}",
                   "phase_ms": {k: round(v, 4) for k, v in phases.items()},
                   "step_algorithmic_gbs": step_bytes / (ms_step * 1e-3) / 1e9,
                   "step_hbm_frac": step_bytes / (ms_step * 1e-3) / 1e9 / peak},
        "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes": algo[dom],
                     "traffic": traffic},
        "e2e": {"value": world * e2e_steps / (e_ms / 1e3), "unit": "grids/s",
                "h2d_bytes_per_step": int(sdf.numel() * 4 + deform.numel() * 4), "d2h_bytes_per_step": 4},
        "gpu_launches": 4 * args.steps,
        "clocks": clk.summary(),
    }
    return res


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
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return
        steps, warmup = max(1, min(args.steps, 3)), max(1, min(args.warmup, 1))
        value, planes, cores, sec = run_cpu(args, steps, warmup, budget_s=20.0)
        out = {"metric": METRIC, "value": value, "unit": "grids/s", "n_gpus": args.gpus, "steps": steps,
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

    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl")
    device = torch.device("cuda", torch.cuda.current_device())
    res = run_ours(args, rank, world, device)
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
