"""bench.py's multi-replica logic on two CPU ranks (gloo): the slowest
rank's time is the job's time, throughput counts every replica's
particles, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    times = [0.75, 1.25]  # rank 1 is the slow replica
    slowest = bench.max_over_ranks(times[rank], world, "cpu")
    out[rank] = (slowest, bench.replica_throughput(1000, world, 4, slowest))
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_count_every_replica():
    world, port = 2, _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for rank in range(world):
        slowest, value = res[rank]
        assert slowest == 1.25
        assert value == pytest.approx(1000 * 2 * 4 / 1.25)


def test_reference_arm_is_silent_off_rank_zero(monkeypatch, capsys):
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = type("A", (), {"scene": "dam_break", "n": 128, "steps": 1, "warmup": 0})()
    bench.run_reference(args)
    assert capsys.readouterr().out == ""


def test_one_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(2.5, 1, "cpu") == 2.5
