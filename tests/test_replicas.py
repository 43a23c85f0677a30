"""Several GPUs run independent replicas (grids are independent: no collective on the
data path).  The benchmark's timing over ranks: each rank's time reduced with MAX,
so every rank reports the slowest one, and the job's throughput counts every
rank's grids.  Two gloo ranks on the CPU, rendezvous on 127.0.0.1."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(10.0 * (rank + 1), world, torch.device("cpu"))
        q.put((rank, ms, bench.job_throughput(world, 30, ms)))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(300)
def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        out = sorted(q.get(timeout=240) for _ in procs)
    finally:
        for p in procs:
            p.join(60)
    assert [p.exitcode for p in procs] == [0, 0]
    assert [o[1] for o in out] == [20.0, 20.0]  # rank 1 took 20 ms: both report it
    assert out[0][2] == out[1][2] == 2 * 30 / 0.020  # 60 grids in 20 ms


def test_one_rank_needs_no_collective():
    import bench

    assert not torch.distributed.is_initialized()
    assert bench.max_over_ranks(7.5, 1, torch.device("cpu")) == 7.5
    assert bench.job_throughput(1, 300, 1260.0) == pytest.approx(238.095, rel=1e-5)
