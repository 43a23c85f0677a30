"""Launch widths change no output (every kernel gives the same bits for any
width), so the autotuner may pick any of them; and the tuner runs end to end on
the GPU (timing, cache file, applying the winner)."""
import pytest
import torch

pytestmark = pytest.mark.gpu

SETTINGS = [{}, {"count_ctas": 1, "emit_ctas": 2, "gather_ctas": 1, "edge_ctas": 3, "zero_share": 900},
            {"fused_ctas": 1, "zero_ctas": 1, "emit_ctas": 1}, {"count_ctas": 2, "zero_share": 1, "zero_ctas": 5}]


@pytest.mark.parametrize("method,kw", [("mc", {}), ("dmc", {"return_quads": True})])
@pytest.mark.parametrize("recompute", [False, True])
def test_launch_widths_change_no_output(cuda_device, method, kw, recompute):
    from diso_gb300 import DiffDMC, DiffMC, tune

    sdf, dfm = tune.synthetic_grid((70, 90, 64), cuda_device, torch.float32)
    out = []
    for setting in SETTINGS:
        mod = DiffMC(torch.float32, recompute=recompute) if method == "mc" else DiffDMC(torch.float32,
                                                                                        recompute=recompute)
        mod._ex.set_launch(setting)
        assert all(mod._ex.launch()[k] == v for k, v in setting.items())
        s = sdf.clone().requires_grad_(True)
        d = dfm.clone().requires_grad_(True)
        for _ in range(2):  # the first call sizes the outputs, the second is the single-call forward
            s.grad = d.grad = None
            v, f = mod(s, d, **kw)
            (v * v).sum().backward()
        out.append((v.detach(), f, s.grad, d.grad))
    for o in out[1:]:
        for a, b in zip(o, out[0]):
            assert torch.equal(a, b)


def test_batch_widths_change_no_output(cuda_device):
    from diso_gb300 import DiffDMCBatch, tune

    grids = [tune.synthetic_grid(sh, cuda_device, torch.float32, seed=i) for i, sh in
             enumerate([(40, 33, 35), (64, 64, 64), (17, 70, 20)])]
    out = []
    for setting in ({}, {"batch_ctas": 1, "gather_ctas": 1, "edge_ctas": 2, "zero_ctas": 1}):
        b = DiffDMCBatch(torch.float32)
        b._bx.ex.set_launch(setting)
        s = [g[0].clone().requires_grad_(True) for g in grids]
        d = [g[1].clone().requires_grad_(True) for g in grids]
        meshes = b(s, d, return_quads=True)
        sum((v * v).sum() for v, _ in meshes).backward()
        out.append(([m for mm in meshes for m in mm], [x.grad for x in s + d]))
    for a, b in zip(out[0][0] + out[0][1], out[1][0] + out[1][1]):
        assert torch.equal(a, b)


def test_tuner_end_to_end(cuda_device, tmp_path, monkeypatch):
    from diso_gb300 import DiffDMC, tune

    monkeypatch.setenv("DISO_TUNE_CACHE", str(tmp_path / "tune.json"))
    mod = DiffDMC(torch.float32, recompute=True)
    entry = tune.tune_module(mod, (96, 96, 96), steps=1)
    assert entry["ms"] <= entry["default_ms"] and entry["trials"] >= 2
    assert mod._ex.launch()["fused_ctas"] == entry["params"]["fused_ctas"]
    # the second call reads the cache and times nothing
    again = tune.tune_module(DiffDMC(torch.float32, recompute=True), (100, 90, 80))
    assert again == entry
