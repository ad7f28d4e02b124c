"""Multi-process (gloo, world_size 2) coverage of the replica path: per-rank seeds and the
max-over-ranks timing that defines the job's aggregate throughput."""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    from cuscan_gb300 import replicas, synthetic

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        seed = replicas.replica_seed(44, rank)
        x = synthetic.vmf_like(n=2000, d=16, clusters=4, seed=seed)
        seconds = 1.0 + rank  # rank 1 is the slow one
        value, worst = replicas.aggregate_throughput(x.shape[0], 3, seconds)
        out[rank] = (seed, float(x[0, 0]), value, worst)
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas_use_distinct_seeds_and_slowest_time():
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    (s0, f0, v0, w0), (s1, f1, v1, w1) = out[0], out[1]
    assert s0 == 44 and s1 == 1044 and f0 != f1
    assert w0 == w1 == 2.0
    assert v0 == v1 == pytest.approx(2 * 2000 * 3 / 2.0)


def test_single_process_is_identity():
    from cuscan_gb300 import replicas

    assert replicas.slowest(1.5) == 1.5
    assert replicas.aggregate_throughput(100, 2, 2.0) == (100.0, 2.0)
