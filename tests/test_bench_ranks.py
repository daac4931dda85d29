"""The bench's multi-rank path on the CPU: two gloo ranks (replicas, no collective on the data path)
take the maximum of their timings and report the whole job's rate; the reference arm runs on rank 0
alone and the other ranks leave at once."""
import os
import socket

import pytest
import torch.multiprocessing as mp

import bench


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # Rank 1 is the slow replica on the device timing, rank 0 on the end-to-end one.
    times = bench.max_over_ranks([1.0 + rank, 5.0 - rank], world)
    out[rank] = (times, bench.whole_job_rate(1 << 20, 5, world, times[0]))
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_replica():
    world, port = 2, free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(rank_main, args=(world, port, out), nprocs=world, join=True)
        got = dict(out)
    for rank in range(world):
        times, rate = got[rank]
        assert times == [2.0, 5.0]
        assert rate == pytest.approx((1 << 20) * bench.ROUNDS * 5 * world / 2.0 / 1e6)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        width, height, steps, warmup, gpus, profile = 64, 32, 1, 1, 2, 0

    def no_sample(*a, **k):
        raise AssertionError("rank 1 must not run the CPU sample")

    monkeypatch.setattr(bench, "CpuSample", no_sample)
    assert bench.run_reference(Args()) == 0
