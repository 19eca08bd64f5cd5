"""Replica bookkeeping of multi-GPU runs, on CPU with two gloo ranks."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from aenet_gb300.replicas import job_rate, max_over_ranks, replica_seed
        units = 1000 * (rank + 1)          # ranks process different batch sizes
        seconds = 0.5 + rank               # and take different times
        out[rank] = (job_rate(units, seconds), max_over_ranks(seconds), replica_seed(4, rank))
    finally:
        dist.destroy_process_group()


def test_two_rank_job_rate_is_total_work_over_slowest_rank():
    world = 2
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    r0, r1 = out[0], out[1]
    assert r0[0] == r1[0] == pytest.approx(3000 / 1.5)
    assert r0[1] == r1[1] == 1.5
    assert (r0[2], r1[2]) == (4, 1004)
