"""bench.py under torchrun: every rank denoises its own copy of the workload
(replicas, no data exchange), the job time is the slowest rank's, and the
reference arm runs on rank 0 alone.  Checked with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from helpers import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank            # rank 1 is the slower replica
    out[rank] = bench.replica_max_ms(ms, world)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_time_is_the_slowest_rank():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    assert out[0] == out[1] == 150.0


def test_single_process_time_is_its_own():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_max_ms(123.5, 1) == 123.5


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        workload = "small"
        steps = 1
        warmup = 0

    assert bench.run_reference(Args()) == 0
    assert capsys.readouterr().out == ""
