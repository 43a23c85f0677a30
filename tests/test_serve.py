"""Serving loop logic without a GPU: admission in arrival order under the HBM
budget, batching by (method, normalize, deform), concurrency across workers, and
a worker that raises failing only its own batch."""
import threading
import time

import pytest

from diso_gb300.serve import Request, Server, Worker, summarize


class FakeWorker(Worker):
    """Sleeps instead of running kernels; records what it was given."""

    log = []
    lock = threading.Lock()

    def setup(self):
        self.fail_rids = getattr(self.server, "fail_rids", set())

    def process(self, batch):
        with FakeWorker.lock:
            FakeWorker.log.append((self.name, [r.rid for r in batch], self.server.in_use))
        time.sleep(0.002 * len(batch))
        if any(r.rid in self.fail_rids for r in batch):
            raise RuntimeError("injected failure")
        t = self.server.now()
        for r in batch:
            r.done = t


def _trace(n, size, gap=0.0005):
    return [Request(rid=i, method=i % 2, shape=(8, 8, 8), make_inputs=None, arrival=i * gap, est_bytes=size)
            for i in range(n)]


def make_server(budget, **kw):
    FakeWorker.log = []
    return Server(device="cpu", hbm_budget=budget, worker_cls=FakeWorker, **kw)


def test_all_requests_complete_and_batches_share_a_key():
    srv = make_server(1e12, max_batch=4, workers=3)
    trace = _trace(40, 10)
    srv.serve(trace)
    srv.close()
    assert all(r.done >= r.arrival for r in trace)
    by_rid = {r.rid: r for r in trace}
    for _, rids, _ in FakeWorker.log:
        assert len(rids) <= 4
        assert len({by_rid[i].key for i in rids}) == 1
    s = summarize(trace)
    assert s["completed"] == 40 and s["p99_ms"] >= s["p50_ms"]


def test_admission_respects_the_budget():
    size = 100
    srv = make_server(3.5 * size, max_batch=8, workers=2)
    trace = _trace(30, size)
    srv.serve(trace)
    srv.close()
    assert srv.peak <= 3.5 * size
    assert max(u for _, _, u in FakeWorker.log) <= 3.5 * size
    # admitted in arrival order
    adm = [r.admitted for r in trace]
    assert adm == sorted(adm)


def test_oversized_request_still_runs_alone():
    srv = make_server(50, max_batch=8, workers=2)
    trace = _trace(3, 80)
    srv.serve(trace)
    srv.close()
    assert all(r.done >= 0 for r in trace) and srv.peak == 80


def test_failing_batch_fails_only_its_requests():
    srv = make_server(1e12, max_batch=1, workers=2)
    srv.fail_rids = {5}
    for w in srv.workers:
        w.fail_rids = {5}
    trace = _trace(12, 1)
    srv.serve(trace)
    srv.close()
    bad = [r.rid for r in trace if r.error]
    assert bad == [5]
    assert all(r.done >= 0 for r in trace)
    assert summarize(trace)["errors"] == 1
