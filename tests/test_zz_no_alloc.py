"""diso_forward_count_static: the forward count phase for callers that cannot
allocate device memory (serving processes whose device memory is reserved at
start-up and may not grow per request, or hosts whose own memory manager owns
the device).

Called through the C ABI and checked against diso_forward_count on the same
inputs, twice in a row, because every call reuses the same static scratch
array and must clear what the previous call left there.  Collected last so that
a run stopping at its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _field(shape, seed):
    rng = np.random.default_rng(seed)
    axes = [np.linspace(-1, 1, n) for n in shape]
    X, Y, Z = np.meshgrid(*axes, indexing="ij")
    s = np.full(shape, np.inf)
    for _ in range(5):
        c = rng.uniform(-0.6, 0.6, 3)
        s = np.minimum(s, np.sqrt((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) - rng.uniform(0.1, 0.3))
    return s + 0.02 * rng.standard_normal(shape)


def _counts_tuple(c):
    return (c.n_verts, c.n_faces, c.sdf_min, c.sdf_max, c.empty, c.n_active_tiles)


@pytest.mark.parametrize("dtype", [torch.float32, torch.float64])
@pytest.mark.parametrize("method", [0, 1])
def test_static_count_matches_extractor_count_twice(cuda_device, method, dtype):
    from diso_gb300 import _native as N

    lib = N.lib()
    ex = N.Extractor(method, dtype)
    stream = N.stream_of(cuda_device)
    np_dtype = np.float32 if dtype == torch.float32 else np.float64
    # two different grids in a row: the second call must not see the first one's state
    for shape, seed in [((70, 45, 90), 1), ((33, 64, 17), 2)]:
        g = torch.tensor(_field(shape, seed).astype(np_dtype), device=cuda_device)
        iso, pad = N.iso_values(0.0, dtype)
        slots = N.Extractor.segment_slots(g.shape)
        # the record is the scanned segment counts, their total and one activity byte per
        # tile; the bytes that pad the last slot are not written, so both start equal
        seg_ref = torch.full((slots,), -1, dtype=torch.int64, device=cuda_device)
        ref = ex.count(g, iso, pad, seg_ref)
        seg = torch.full((slots,), -1, dtype=torch.int64, device=cuda_device)
        out = N.Counts()
        rc = lib.diso_forward_count_static(method, N.dtype_tag(dtype), N.ptr(g), *g.shape, iso, pad, N.ptr(seg),
                                           stream, ctypes.byref(out))
        assert rc == 0, lib.diso_last_error()
        torch.cuda.synchronize()
        # integer outputs: exact (the tolerance of every count and index in this suite)
        assert _counts_tuple(out) == _counts_tuple(ref)
        c0, c1, c2 = (n + 1 for n in shape)
        nzc = (c2 + 31) // 32
        nseg = c0 * c1 * nzc
        ntiles = ((c0 + 3) // 4) * ((c1 + 7) // 8) * nzc
        assert torch.equal(seg[:nseg + 1], seg_ref[:nseg + 1])
        flags = seg[nseg + 1:].view(torch.uint8)[:ntiles]
        assert torch.equal(flags, seg_ref[nseg + 1:].view(torch.uint8)[:ntiles])
        assert int(flags.sum()) == out.n_active_tiles
        assert torch.equal(seg, seg_ref)


def test_static_count_rejects_oversized_grids(cuda_device):
    from diso_gb300 import _native as N

    lib = N.lib()
    small = torch.zeros(8, device=cuda_device)
    seg = torch.zeros(8, dtype=torch.int64, device=cuda_device)
    out = N.Counts()
    # 400^3 has 101 x 51 x 13 = 66963 tiles: rejected before any GPU work
    rc = lib.diso_forward_count_static(0, N.F32, N.ptr(small), 400, 400, 400, 0.0, 1.0, N.ptr(seg),
                                       N.stream_of(cuda_device), ctypes.byref(out))
    assert rc == 1
    assert b"too large for diso_forward_count_static" in lib.diso_last_error()
