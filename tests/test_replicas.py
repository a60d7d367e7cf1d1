"""The N-GPU bench path on CPU: two gloo ranks, each with its own replica
time; the job time is the slowest rank's and the throughput counts every
rank's units (the contact path has no data exchange between GPUs)."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, rank, world)
        ms = [10.0, 25.0][rank]  # the second rank is slower
        m = bench.max_over_ranks(ms, world, device="cpu")
        out[rank] = (m, bench.replica_throughput(1000, m, world))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time():
    port = _free_port()
    with mp.Manager() as man:
        out = man.dict()
        mp.spawn(_rank, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    for rank in (0, 1):
        m, v = res[rank]
        assert m == 25.0
        assert v == pytest.approx(2 * 1000 / 0.025)


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.max_over_ranks(12.5, 1, device="cpu") == 12.5
    assert bench.replica_throughput(3776, 2.0, 1) == pytest.approx(3776 / 0.002)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    # under torchrun the CPU reference arm runs once, on rank 0; the other
    # ranks return at once without work
    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert bench.run_reference(None) is None
