"""Host arithmetic behind the benchmark's roofline (no GPU): the algorithmic bytes per
launch that `roofline.achieved` divides by the kernel's time, and the committed DRAM
traffic summary that `roofline.traffic` quotes, which belongs to one workload size."""
import bench

N = 512
VOL = N ** 3
NSEG = (N + 1) ** 2 * ((N + 1 + 31) // 32)
# the 512^3 benchmark field's DMC mesh and its point tiles with a crossing nearby
VERTS, QUADS, ACTIVE_PTS = 3_563_952, 3_301_242, 11_634 * 1024


def test_fused_backward_bytes_at_512():
    b = bench.kernel_bytes(VOL, NSEG, VERTS, QUADS, 4, 0.0, ACTIVE_PTS)
    s = 4
    # active tiles' SDF in and both gradients out, deform at the edges' ends, dL/dverts,
    # the zeros of every other point's gradients
    expect = ACTIVE_PTS * 5 * s + 6 * s * QUADS + 3 * s * VERTS + (VOL - ACTIVE_PTS) * 4 * s
    assert b["fused_bwd"] == expect == 2_317_133_744


def test_step_bytes_are_the_sum_of_the_dense_and_sparse_terms():
    s = 4
    step = VOL * s * (3 + 3) + 4 * QUADS * 3 * s + 2 * VERTS * 3 * s + 8 * QUADS * 4
    assert 3.5e9 < step < 3.6e9  # the 3.57 GB the step's HBM fraction is taken of


def test_stored_mode_zero_shares_add_up():
    z = 0.35
    b = bench.kernel_bytes(VOL, NSEG, VERTS, QUADS, 4, z, ACTIVE_PTS)
    zeros = VOL * 4 * 4
    count_own = VOL * 4 + NSEG * 8
    emit_own = 2 * QUADS * 4 * 4 + VERTS * 3 * 4 + QUADS * 4 * 8 + QUADS * (8 + 16) + VERTS
    assert abs((b["count"] - count_own) + (b["emit"] - emit_own) - zeros) < 1e-3 * zeros


def test_traffic_summary_is_read_for_its_own_size_only():
    t = bench.read_profile_traffic("fused_bwd", 512)
    assert t is not None and 1.5e9 < t < 2.5e9
    assert bench.read_profile_traffic("fused_bwd", 256) is None
    assert bench.read_profile_traffic("no_such_kernel", 512) is None
