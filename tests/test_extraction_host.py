"""Host logic of the extraction modules that needs no GPU: the check of the forward
that a recompute-mode backward runs again, and argument checks of batches."""
import pytest
import torch

from diso_gb300 import _native as N
from diso_gb300.batch import extract_batch
from diso_gb300.extraction import _recompute


@pytest.fixture(scope="module", autouse=True)
def native_library():
    # segment_slots is plain arithmetic in the library (no GPU needed); build it if absent
    from diso_gb300.build import build

    build()


class _FakeExtractor:
    """Stands in for the native extractor: its forward reports fixed counts."""

    method, dtype = N.MC, torch.float32

    def __init__(self, n_verts, n_faces, emitted=1):
        self.counts = (n_verts, n_faces, emitted)
        self.calls = []

    def zero_grads(self, gs, gd):
        self.calls.append("zero_grads")

    def record_slots(self, n_verts, n_faces):
        return 8 * (n_verts + n_faces)

    def forward(self, g, d, iso, pad, seg, normalize, verts, faces, record):
        self.calls.append("forward")
        assert verts.shape == (5, 3) and faces.shape == (3, 3) and record.numel() == 64
        c = N.Counts()
        c.n_verts, c.n_faces, c.emitted = self.counts
        return c


def test_recompute_runs_the_forward_after_zeroing_new_gradient_buffers():
    ex = _FakeExtractor(5, 3)
    g = torch.zeros(4, 4, 4)
    seg, record, gs, gd = _recompute(ex, g, torch.zeros(4, 4, 4, 3), 0.0, 1.0, True, 5, 3)
    assert ex.calls == ["zero_grads", "forward"]
    assert gs.shape == g.shape and gd.shape == (4, 4, 4, 3) and record.numel() == 64
    assert seg.numel() == N.Extractor.segment_slots(g.shape)
    _, _, _, gd = _recompute(_FakeExtractor(5, 3), g, None, 0.0, 1.0, True, 5, 3)
    assert gd is None


@pytest.mark.parametrize("counts", [(6, 3, 1), (5, 4, 1), (5, 3, 0)])
def test_recompute_refuses_another_mesh(counts):
    # a grid changed between the forward and the backward gives other counts (or
    # does not fit the forward's sizes): the backward must not use that record
    with pytest.raises(RuntimeError, match="another mesh"):
        _recompute(_FakeExtractor(*counts), torch.zeros(4, 4, 4), None, 0.0, 1.0, True, 5, 3)


def test_batch_isovalue_count_must_match_the_grids():
    grids = [torch.zeros(3, 3, 3), torch.zeros(3, 3, 3)]
    with pytest.raises(RuntimeError, match="1 isovalues for 2 grids"):
        extract_batch(object(), grids, isovalue=[0.0])
