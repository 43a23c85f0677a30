"""Bounded device-side waits end in an error status, not a hang.  The segment
scan's look-back is run with a predecessor whose flag is never published
(diso_scan_wait_probe) and a small poll limit: the call must return DISO_ERR_SCAN
with the scan's message, and the same extractor must then extract as before."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("limit", [1, 64, 4096])
def test_lookback_wait_gives_up_with_an_error(cuda_device, limit):
    from diso_gb300 import DiffMC
    from diso_gb300 import _native as N

    mod = DiffMC(torch.float32)
    a = np.linspace(-1, 1, 40)
    X, Y, Z = np.meshgrid(a, a, a, indexing="ij")
    sdf = torch.tensor((np.sqrt(X * X + Y * Y + Z * Z) - 0.5).astype(np.float32), device=cuda_device)
    with torch.no_grad():
        v0, f0 = mod(sdf)
    rc = N.lib().diso_scan_wait_probe(mod._ex._h, limit, N.stream_of(cuda_device))
    assert rc == 3  # DISO_ERR_SCAN
    assert b"look-back wait gave up" in N.lib().diso_last_error()
    with torch.no_grad():
        v1, f1 = mod(sdf)
    assert torch.equal(v0, v1) and torch.equal(f0, f1)
