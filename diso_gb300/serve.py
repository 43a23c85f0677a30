"""Serving: a request loop with continuous batching and HBM-budget admission.

Each request is one extraction + backward (MC or DMC quads, any grid size).  The
dispatcher admits requests in arrival order while their estimated device
memory fits the budget, keeps their grids and meshes on the device, and hands
batches of waiting requests of one method to idle workers.  Every worker owns a
CUDA stream and its own batch extractors, so a batch that arrives while others
are on the GPU is admitted and runs concurrently as soon as a worker and memory
are free (continuous batching, not a queue in front of one call).  Results are
bit-identical to the same request run alone through DiffMC / DiffDMC (the
kernels are the same and deterministic).
"""
from __future__ import annotations

import threading
import time
from collections import deque
from dataclasses import dataclass, field

import torch

from . import _native as N
from .batch import _Batch, _grids, record_slots


@dataclass
class Request:
    """One extraction + backward.  `make_inputs(device, stream)` returns (sdf,
    deform or None, dL/dverts generator) on the device; `arrival` is seconds
    after the start of the trace."""

    rid: int
    method: int
    shape: tuple
    make_inputs: object
    arrival: float = 0.0
    isovalue: float = 0.0
    normalize: bool = True
    has_deform: bool = True
    est_bytes: int = 0
    # filled by the server
    admitted: float = -1.0
    done: float = -1.0
    verts: torch.Tensor = None
    faces: torch.Tensor = None
    grad_sdf: torch.Tensor = None
    grad_deform: torch.Tensor = None
    error: str = None

    @property
    def latency(self):
        return self.done - self.arrival

    @property
    def key(self):
        """Requests batched together agree on these."""
        return (self.method, self.normalize, self.has_deform)


def estimate_bytes(shape, dtype=torch.float32, deform=True, dense=False):
    """Device memory of a request: grid, deform, both gradients, the per-call record
    and its mesh (dense fields cross on about half of all edges)."""
    n = shape[0] * shape[1] * shape[2]
    s = torch.tensor([], dtype=dtype).element_size()
    grid = n * s * (1 + (3 if deform else 0)) * 2
    cells = (shape[0] + 1) * (shape[1] + 1) * (shape[2] + 1)
    crossings = 1.5 * cells if dense else 40.0 * cells ** (2.0 / 3.0)
    mesh = crossings * (3 * s + 4 * 8 + 3 * s)  # verts, quads / triangles, dL/dverts
    return int(grid + cells / 4 + mesh)


class Worker(threading.Thread):
    """Runs batches handed over by the server; subclasses replace setup() / process()
    (the tests use a worker without a GPU to exercise admission and dispatch)."""

    def __init__(self, server, idx):
        super().__init__(daemon=True, name=f"diso-serve-{idx}")
        self.server = server
        self.inbox = deque()
        self.wake = threading.Event()
        self.busy = False
        self.setup()

    def setup(self):
        self.stream = torch.cuda.Stream(self.server.device)
        self.bx = {m: _Batch(m, self.server.dtype) for m in (N.MC, N.DMC)}

    def run(self):
        srv = self.server
        while not srv.stopping:
            self.wake.wait(0.05)
            self.wake.clear()
            while self.inbox:
                batch = self.inbox.popleft()
                try:
                    self.process(batch)
                except Exception as e:  # a failing batch fails its requests, not the server
                    for r in batch:
                        r.error = repr(e)
                        r.done = srv.now()
                finally:
                    for r in batch:
                        srv.release(r)
                    with srv.lock:
                        srv.completed += len(batch)
                    self.busy = False
                    srv.poke.set()

    def process(self, batch):
        # requests of one batch share method, normalize and whether they carry a deform
        srv = self.server
        dev = srv.device
        with torch.cuda.device(dev), torch.cuda.stream(self.stream):
            method = batch[0].method
            bx = self.bx[method]
            ins = [r.make_inputs(dev) for r in batch]
            sdfs = [x[0] for x in ins]
            has_def = ins[0][1] is not None
            defs = [x[1] for x in ins] if has_def else None
            gs = [torch.empty_like(s) for s in sdfs]
            gd = [torch.empty_like(d) for d in defs] if has_def else None
            isos = [r.isovalue for r in batch]
            grids = _grids(sdfs, defs, isos, srv.dtype, gs, gd)
            record = torch.empty(record_slots(grids), dtype=torch.int64, device=dev)
            bx.prepare(grids, record, dev)
            bx.count(dev)
            res = bx.results(len(batch), dev)
            n = len(batch)
            nv = int(res.voff[n - 1] + res.counts[n - 1].n_verts)
            nf = int(res.foff[n - 1] + res.counts[n - 1].n_faces)
            width = 3 if method == N.MC else 4
            verts = torch.empty((nv, 3), dtype=srv.dtype, device=dev)
            faces = torch.empty((nf, width), dtype=torch.int64, device=dev)
            edges = bx.edge_record(nv, nf, dev)
            bx.emit(batch[0].normalize, verts, faces, dev, edges)
            gv = torch.empty_like(verts)
            for i, (r, x) in enumerate(zip(batch, ins)):
                v0, c = int(res.voff[i]), res.counts[i]
                gv[v0:v0 + c.n_verts] = x[2](c.n_verts)
            bx.backward(batch[0].normalize, False, gv, edges, nv, nf, dev)
            self.stream.synchronize()
            t = srv.now()
            for i, r in enumerate(batch):
                c = res.counts[i]
                v0, f0 = int(res.voff[i]), int(res.foff[i])
                iso = N.iso_values(r.isovalue, srv.dtype)[0]
                if c.sdf_min >= iso or c.sdf_max <= iso:
                    r.verts = verts[:0]
                    r.faces = torch.zeros((0, width), dtype=torch.int32, device=dev)
                else:
                    r.verts = verts[v0:v0 + c.n_verts]
                    r.faces = faces[f0:f0 + c.n_faces]
                r.grad_sdf = gs[i]
                r.grad_deform = gd[i] if has_def else None
                r.done = t


class Server:
    """Continuous-batching extraction server on one GPU."""

    def __init__(self, device="cuda", dtype=torch.float32, hbm_budget=60e9, max_batch=32, workers=2,
                 keep_results=False, worker_cls=None):
        self.device = torch.device(device)
        self.dtype = dtype
        self.budget = float(hbm_budget)
        self.max_batch = max_batch
        self.keep = keep_results
        self.in_use = 0.0
        self.peak = 0.0
        self.completed = 0
        self.lock = threading.Lock()
        self.poke = threading.Event()
        self.stopping = False
        self.t0 = time.perf_counter()
        self.workers = [(worker_cls or Worker)(self, i) for i in range(workers)]
        for w in self.workers:
            w.start()

    def now(self):
        return time.perf_counter() - self.t0

    def release(self, r):
        with self.lock:
            self.in_use -= r.est_bytes
        if not self.keep:
            r.verts = r.faces = r.grad_sdf = r.grad_deform = None

    def close(self):
        self.stopping = True
        for w in self.workers:
            w.wake.set()
            w.join(timeout=5)

    def serve(self, trace, realtime=True):
        """Run `trace` (Requests sorted by arrival); returns when all are done."""
        self.t0 = time.perf_counter()
        with self.lock:
            self.completed = 0
        pending = deque(trace)
        waiting = deque()
        total = len(trace)
        while True:
            # cleared before looking, so a completion signalled while we look is not lost
            self.poke.clear()
            now = self.now()
            # admission: arrival order, while the budget allows
            blocked = False
            while pending and (pending[0].arrival <= now or not realtime):
                r = pending[0]
                with self.lock:
                    fits = self.in_use + r.est_bytes <= self.budget or self.in_use == 0
                    if fits:
                        self.in_use += r.est_bytes
                        self.peak = max(self.peak, self.in_use)
                if not fits:
                    blocked = True
                    break
                pending.popleft()
                r.admitted = now
                waiting.append(r)
            # dispatch: the oldest waiting request's kind, up to max_batch of that kind
            for w in self.workers:
                if not waiting:
                    break
                if w.busy:
                    continue
                key = waiting[0].key
                batch, rest = [], deque()
                while waiting and len(batch) < self.max_batch:
                    r = waiting.popleft()
                    (batch if r.key == key else rest).append(r)
                waiting.extendleft(reversed(rest))
                w.busy = True
                w.inbox.append(batch)
                w.wake.set()
            with self.lock:
                finished = self.completed == total
            if finished:
                break
            # sleep until the next arrival, or until a worker finishes (which frees memory
            # and a worker); never spin, the workers need the interpreter
            if pending and not blocked and realtime:
                timeout = max(0.0, pending[0].arrival - self.now())
            else:
                timeout = 0.05
            self.poke.wait(timeout)
        return trace


def summarize(trace, t_first=None):
    lat = sorted(r.latency for r in trace if r.error is None)
    errs = sum(1 for r in trace if r.error is not None)
    if not lat:
        return {"completed": 0, "errors": errs}
    start = min(r.arrival for r in trace) if t_first is None else t_first
    end = max(r.done for r in trace)

    def pct(p):
        return lat[min(len(lat) - 1, int(round(p / 100.0 * (len(lat) - 1))))] * 1e3

    return {"completed": len(lat), "errors": errs, "p50_ms": pct(50), "p99_ms": pct(99),
            "grids_per_s": len(lat) / max(end - start, 1e-9), "wall_s": end - start}


def serve_plain(trace, device="cuda", dtype=torch.float32, realtime=True):
    """The baseline: the same requests, one at a time in arrival order, each through
    the plain single-grid module (a per-request call), on the default stream."""
    from .extraction import extract

    dev = torch.device(device)
    ex = {m: N.Extractor(m, dtype) for m in (N.MC, N.DMC)}
    t0 = time.perf_counter()
    with torch.cuda.device(dev):
        for r in trace:
            if realtime:
                while time.perf_counter() - t0 < r.arrival:
                    time.sleep(0.0002)
            sdf, dfm, grad = r.make_inputs(dev)
            sdf.requires_grad_(True)
            if dfm is not None:
                dfm.requires_grad_(True)
            v, f = extract(ex[r.method], sdf, dfm, r.isovalue, r.normalize, True)
            if v.requires_grad:
                torch.autograd.backward(v, grad(v.shape[0]))
            torch.cuda.synchronize()
            r.done = time.perf_counter() - t0
    return trace
