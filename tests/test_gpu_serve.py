"""Served requests (continuous batching, HBM-budget admission, two concurrent
workers) give exactly the result of the same request run alone."""
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_each_result_same_alone_and_in_the_mix(cuda_device):
    from bench import request_inputs
    from diso_gb300 import _native as N
    from diso_gb300.extraction import extract
    from diso_gb300.serve import Request, Server, estimate_bytes

    shapes = [(24, 24, 24), (40, 33, 35), (16, 16, 16), (48, 48, 48), (31, 20, 17), (64, 64, 64)] * 3
    kinds = ["sphere", "random", "box"]
    trace = []
    for i, sh in enumerate(shapes):
        kind = kinds[i % 3]
        trace.append(Request(rid=i, method=(i // 2) % 2, shape=sh, arrival=0.002 * i,
                             make_inputs=request_inputs(100 + i, sh, kind),
                             est_bytes=estimate_bytes(sh, dense=kind == "random")))
    budget = 3.5 * max(r.est_bytes for r in trace)
    srv = Server(cuda_device, hbm_budget=budget, max_batch=4, workers=2, keep_results=True)
    srv.serve(trace)
    srv.close()
    assert srv.peak <= budget
    assert all(r.error is None for r in trace), [r.error for r in trace if r.error]
    ex = {m: N.Extractor(m, torch.float32) for m in (0, 1)}
    for r in trace:
        sdf, dfm, grad = r.make_inputs(cuda_device)
        sdf.requires_grad_(True)
        dfm.requires_grad_(True)
        v, f = extract(ex[r.method], sdf, dfm, 0.0, True, True)
        assert torch.equal(r.faces, f) and torch.equal(r.verts, v), f"request {r.rid}: mesh differs"
        if v.shape[0]:
            torch.autograd.backward(v, grad(v.shape[0]))
            assert torch.equal(r.grad_sdf, sdf.grad) and torch.equal(r.grad_deform, dfm.grad), \
                f"request {r.rid}: gradients differ"
