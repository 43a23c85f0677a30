"""Host logic of the extraction modules that needs no GPU: argument checks of
batches."""
import pytest
import torch

from diso_gb300.batch import extract_batch


@pytest.fixture(scope="module", autouse=True)
def native_library():
    # segment_slots is plain arithmetic in the library (no GPU needed); build it if absent
    from diso_gb300.build import build

    build()


def test_batch_isovalue_count_must_match_the_grids():
    grids = [torch.zeros(3, 3, 3), torch.zeros(3, 3, 3)]
    with pytest.raises(RuntimeError, match="1 isovalues for 2 grids"):
        extract_batch(object(), grids, isovalue=[0.0])
