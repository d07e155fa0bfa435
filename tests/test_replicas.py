"""The multi-GPU path runs independent replicas (the particle path does not shard).
Its only exchange is the final throughput reduction, checked here with two gloo
ranks on CPU: value = units of all ranks / the slowest rank's time."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pairs_gb300.replicas import job_throughput


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units = 1000.0 * (rank + 1)            # rank 0: 1000 atom-steps in 10 ms, rank 1: 2000 in 40 ms
    ms = 10.0 * (rank + 1) ** 2
    value, ms_max = job_throughput(units, ms, dist)
    out[rank] = (value, ms_max)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_job_throughput():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        value, ms = out[r]
        assert ms == 40.0
        assert abs(value - 3000.0 / 0.040) < 1e-6


def test_single_process_throughput():
    value, ms = job_throughput(500.0, 5.0, None)
    assert ms == 5.0 and abs(value - 1e5) < 1e-9
